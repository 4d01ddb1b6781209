// Batched QR / polar over a list of independent, uneven blocks (the symmetry
// sectors of a block-sparse tensor), GB300 native.
//
// The reference has no batched API: a caller loops over blocks and calls
// qr_compact! / left_polar! once per block (the symmetry sectors of a
// block-sparse tensor, an orthogonalisation sweep).  Here
// one call takes the whole work list:
//  * blocks are ordered by estimated flops (longest first) and dealt to the
//    least-loaded of the internal streams (LPT schedule), so large
//    blocks keep their multi-CTA kernels while small blocks fill the
//    remaining SMs concurrently;
//  * the internal streams fork from and join back into the caller's stream
//    with events, so the whole batch is one stream-ordered unit that a
//    caller can capture into a CUDA graph.  The streams and events belong
//    to the calling host thread and the current device (created by that
//    thread's first batched call on that device, which must therefore
//    precede any capture there): calls from several threads never share an
//    event, and a call on another device never uses this device's streams;
//  * each stream owns a slice of the caller's workspace sized for the
//    largest block it runs; every block writes its own mak_info record;
//  * batched polar runs the Newton iteration in its fixed-iteration mode
//    (maxiter iterations, no host synchronization).
#include <algorithm>
#include <mutex>
#include <vector>

#include "internal.h"

namespace mak {

// internal streams: MAK_BATCH_STREAMS (default 32 = kMaxBatchStreams).
// Measured on the 300 uneven blocks (graph replay, mixed polar): 8 / 16 / 32
// streams 2.09 / 1.80 / 1.77 s with the tensor-core Gauss-Jordan updates
// from n^2 128 >= 2^25; the blocks' chains of latency-bound panels overlap
// better the more streams carry them.
constexpr int kMaxBatchStreams = 32;
static int batch_streams() {
  return (int)tuning(TUNE_BATCH_STREAMS);
}

struct StreamPool {
  cudaStream_t s[kMaxBatchStreams];
  cudaEvent_t fork, join[kMaxBatchStreams];
  int state = 0;  // 0 not created, 1 ready, -1 failed
};

// the calling thread's pool on the current device (nullptr on failure)
static StreamPool* pool() {
  static thread_local StreamPool p[kMaxDevices];
  StreamPool& q = p[current_device()];
  if (q.state == 0) {
    bool ok = true;
    for (int i = 0; i < kMaxBatchStreams; i++) {
      ok &= cudaStreamCreateWithFlags(&q.s[i], cudaStreamNonBlocking) == cudaSuccess;
      ok &= cudaEventCreateWithFlags(&q.join[i], cudaEventDisableTiming) == cudaSuccess;
    }
    ok &= cudaEventCreateWithFlags(&q.fork, cudaEventDisableTiming) == cudaSuccess;
    q.state = ok ? 1 : -1;
  }
  return q.state == 1 ? &q : nullptr;
}

enum { BATCH_QR = 0, BATCH_POLAR = 1 };

template <class T>
static int item_run(int kind, const mak_batch_item& it, const void* opts, Arena& ar,
                    mak_info* info, cudaStream_t st) {
  const int64_t m = it.m, n = it.n;
  if (kind == BATCH_QR) {
    const mak_qr_opts* o = (const mak_qr_opts*)opts;
    const int64_t k = m < n ? m : n;
    return qr_run<T>(st, m, n, (T*)it.A, it.lda, (T*)it.Q, it.ldq, k, (T*)it.R, it.ldr, k,
                     o->positive, o->blocksize, o->precision, ar, info);
  }
  const mak_polar_opts* o = (const mak_polar_opts*)opts;
  // fixed-iteration mode (negative tol); default tol = eps(real T)^(2/3)
  const double dtol = sizeof(real_t<T>) == 8 ? 3.6700562101601e-11 : 2.4214387e-5;
  const double tol = -(o->tol > 0 ? o->tol : dtol);
  return polar_newton_run<T>(st, m, n, (T*)it.A, it.lda, (T*)it.Q, it.ldq, (T*)it.R, it.ldr,
                             o->maxiter, tol, o->precision, ar, info);
}

static int item_dispatch(int kind, const mak_batch_item& it, const void* opts, Arena& ar,
                         mak_info* info, cudaStream_t st) {
  switch (it.dtype) {
    case MAK_F64: return item_run<double>(kind, it, opts, ar, info, st);
    case MAK_C64: return item_run<zcomplex>(kind, it, opts, ar, info, st);
    case MAK_F32: return item_run<float>(kind, it, opts, ar, info, st);
    case MAK_C32: return item_run<ccomplex>(kind, it, opts, ar, info, st);
    default: return MAK_ERR_UNSUPPORTED;
  }
}

static double item_flops(int kind, const mak_batch_item& it) {
  const double m = (double)it.m, n = (double)it.n;
  const double c = (it.dtype == MAK_C64 || it.dtype == MAK_C32) ? 4.0 : 1.0;
  const double k = m < n ? m : n;
  double f = c * (4.0 * m * k * k - 4.0 * k * k * k / 3.0);
  if (kind == BATCH_POLAR) f += c * 10.0 * 2.0 * n * n * n;
  return f + 1e6;  // launch overheads dominate tiny blocks
}

struct Plan {
  std::vector<int> owner;            // stream of each item (-1: the one-CTA small-block launch)
  std::vector<int> small;            // items factored by the one-CTA small-block kernel
  std::vector<size_t> ws_item;       // workspace of each item
  size_t ws_stream[kMaxBatchStreams];   // slice size per stream
  size_t off[kMaxBatchStreams];
  size_t total;
  size_t extra_off = 0;              // a region after the slices (pullback ranks)
};

static int plan(int kind, const mak_batch_item* items, int nitems, const void* opts, Plan& p) {
  p.owner.assign(nitems, 0);
  p.ws_item.assign(nitems, 0);
  p.small.clear();
  // blocks that fit one CTA's shared memory go to one persistent launch
  const int small_cap = kind == BATCH_QR ? small_qr_cap() : small_polar_cap();
  std::vector<int> order;
  order.reserve(nitems);
  for (int i = 0; i < nitems; i++) {
    if (kind == BATCH_QR ? small_qr_fits(items[i], small_cap)
                         : small_polar_fits(items[i], small_cap)) {
      p.owner[i] = -1;
      p.small.push_back(i);
      continue;
    }
    order.push_back(i);
    Arena meas(nullptr, 0);
    mak_batch_item probe = items[i];
    probe.A = probe.Q = probe.R = nullptr;
    if (kind == BATCH_POLAR && items[i].R != nullptr) probe.R = (void*)16;  // P wanted
    int rc = item_dispatch(kind, probe, opts, meas, nullptr, 0);
    if (rc != 0) return rc;
    p.ws_item[i] = meas.off + 512;
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return item_flops(kind, items[a]) > item_flops(kind, items[b]);
  });
  double load[kMaxBatchStreams] = {0};
  const int ns = batch_streams();
  for (int s = 0; s < kMaxBatchStreams; s++) p.ws_stream[s] = 0;
  for (int i : order) {
    int best = 0;
    for (int s = 1; s < ns; s++)
      if (load[s] < load[best]) best = s;
    p.owner[i] = best;
    load[best] += item_flops(kind, items[i]);
    if (p.ws_item[i] > p.ws_stream[best]) p.ws_stream[best] = p.ws_item[i];
  }
  p.total = 0;
  for (int s = 0; s < kMaxBatchStreams; s++) {
    p.off[s] = p.total;
    p.total += align_up(p.ws_stream[s], 256);
  }
  return 0;
}

static int batched(int kind, const mak_batch_item* items, int nitems, const void* opts,
                   void* work, size_t work_bytes, mak_info* infos, mak_stream_t stream) {
  if (items == nullptr && nitems > 0) return -1;
  if (nitems < 0) return -2;
  for (int i = 0; i < nitems; i++) {
    const mak_batch_item& it = items[i];
    if (it.m < 0 || it.n < 0 || it.lda < (it.m > 1 ? it.m : 1) || it.ldq < (it.m > 1 ? it.m : 1))
      return -1;
    if (kind == BATCH_POLAR && it.n > it.m) return -1;
    if (it.dtype < MAK_F64 || it.dtype > MAK_C32) return -1;
  }
  if (opts == nullptr) return -3;
  Plan p;
  MAK_TRY(plan(kind, items, nitems, opts, p));
  if (work == nullptr && p.total > 0) return -4;
  if (p.total > work_bytes) return -5;
  if (infos == nullptr && nitems > 0) return -6;
  if (nitems == 0) return 0;
  StreamPool* pp = pool();
  if (pp == nullptr) return MAK_ERR_CUDA;
  StreamPool& sp = *pp;
  cudaStream_t st = (cudaStream_t)stream;
  MAK_CUDA_TRY(cudaEventRecord(sp.fork, st));
  const int ns = batch_streams();
  for (int s = 0; s < ns; s++) MAK_CUDA_TRY(cudaStreamWaitEvent(sp.s[s], sp.fork, 0));
  // issue in schedule order so that each stream starts with its largest block
  std::vector<int> order(nitems);
  for (int i = 0; i < nitems; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return item_flops(kind, items[a]) > item_flops(kind, items[b]);
  });
  int rc_all = 0;
  if (!p.small.empty()) {
    // the small blocks: one persistent launch on the caller's stream, which
    // runs beside the internal streams (forked above, joined below)
    if (kind == BATCH_QR) {
      const mak_qr_opts* o = (const mak_qr_opts*)opts;
      rc_all = small_qr_launch(st, items, p.small.data(), (int)p.small.size(), o->positive,
                               infos, small_qr_cap());
    } else {
      const mak_polar_opts* o = (const mak_polar_opts*)opts;
      rc_all = small_polar_launch(st, items, p.small.data(), (int)p.small.size(), o->maxiter,
                                  o->tol, infos, small_polar_cap());
    }
  }
  {
    // the batch's streams already overlap the blocks (no look-ahead), and a
    // quarter of the SMs per split product lets several blocks' persistent
    // tensor-core grids and native kernels share the GPU
    ThreadSettingsScope settings(false, (int)tuning(TUNE_BATCH_GEMM_CTAS));
    for (int i : order) {
      const int s = p.owner[i];
      if (s < 0) continue;  // in the small-block launch
      Arena ar((char*)work + p.off[s], p.ws_stream[s]);
      int rc = info_reset(sp.s[s], infos + i);
      if (rc == 0) rc = item_dispatch(kind, items[i], opts, ar, infos + i, sp.s[s]);
      if (rc != 0 && rc_all == 0) rc_all = rc;
    }
  }
  for (int s = 0; s < ns; s++) {
    MAK_CUDA_TRY(cudaEventRecord(sp.join[s], sp.s[s]));
    MAK_CUDA_TRY(cudaStreamWaitEvent(st, sp.join[s], 0));
  }
  return rc_all;
}

static int batched_ws(int kind, const mak_batch_item* items, int nitems, const void* opts,
                      size_t* bytes) {
  if (bytes == nullptr) return -4;
  if (items == nullptr && nitems > 0) return -1;
  if (opts == nullptr) return -3;
  Plan p;
  MAK_TRY(plan(kind, items, nitems, opts, p));
  *bytes = p.total + 256;
  return 0;
}

// ------------------------------------------------------------- pullbacks --
// Batched reverse rules over the same kind of block list (the pullbacks of a
// whole block-sparse tensor or orthogonalisation sweep in one call).  The QR
// pullback's product shapes depend on each block's numerical rank: the ranks
// of all blocks are computed first and read with ONE host synchronization,
// then every block's pullback is queued without further ones.  The polar
// pullback's Sylvester sign iteration runs a fixed number of steps and stops
// on the device, so that call synchronizes nothing.
enum { BATCH_QR_PB = 2, BATCH_POLAR_PB = 3 };

static int sign_fixed_iters() {
  return (int)tuning(TUNE_SIGN_FIXED_ITERS);
}

template <class T>
static int pb_item_run(int kind, const mak_batch_pullback_item& it, const mak_pullback_opts& o,
                       Arena& ar, mak_info* info, cudaStream_t st, int known_p) {
  if (kind == BATCH_QR_PB)
    return qr_pullback_run<T>(st, it.m, it.n, 0, (T*)it.dA, it.ldda, (const T*)it.F1, it.ld1,
                              (const T*)it.F2, it.ld2, (const T*)it.dF1, it.ldd1,
                              (const T*)it.dF2, it.ldd2, o.rank_atol, o.gauge_atol, o.precision,
                              ar, info, known_p);
  return polar_pullback_run<T>(st, it.m, it.n, (T*)it.dA, it.ldda, (const T*)it.F1, it.ld1,
                               (const T*)it.F2, it.ld2, (const T*)it.dF1, it.ldd1,
                               (const T*)it.dF2, it.ldd2, -sign_fixed_iters(), o.precision, ar,
                               info);
}
static int pb_dispatch(int kind, const mak_batch_pullback_item& it, const mak_pullback_opts& o,
                       Arena& ar, mak_info* info, cudaStream_t st, int known_p) {
  switch (it.dtype) {
    case MAK_F64: return pb_item_run<double>(kind, it, o, ar, info, st, known_p);
    case MAK_C64: return pb_item_run<zcomplex>(kind, it, o, ar, info, st, known_p);
    case MAK_F32: return pb_item_run<float>(kind, it, o, ar, info, st, known_p);
    case MAK_C32: return pb_item_run<ccomplex>(kind, it, o, ar, info, st, known_p);
    default: return MAK_ERR_UNSUPPORTED;
  }
}
static int rank_dispatch(const mak_batch_pullback_item& it, const mak_pullback_opts& o, Arena& ar,
                         cudaStream_t st, int* p_out) {
  const int64_t k = it.m < it.n ? it.m : it.n;
  switch (it.dtype) {
    case MAK_F64: return qr_rank_run<double>(st, k, it.n, (const double*)it.F2, it.ld2, o.rank_atol, ar, p_out);
    case MAK_C64: return qr_rank_run<zcomplex>(st, k, it.n, (const zcomplex*)it.F2, it.ld2, o.rank_atol, ar, p_out);
    case MAK_F32: return qr_rank_run<float>(st, k, it.n, (const float*)it.F2, it.ld2, o.rank_atol, ar, p_out);
    case MAK_C32: return qr_rank_run<ccomplex>(st, k, it.n, (const ccomplex*)it.F2, it.ld2, o.rank_atol, ar, p_out);
    default: return MAK_ERR_UNSUPPORTED;
  }
}
static double pb_flops(int kind, const mak_batch_pullback_item& it) {
  const double m = (double)it.m, n = (double)it.n;
  const double c = (it.dtype == MAK_C64 || it.dtype == MAK_C32) ? 4.0 : 1.0;
  const double k = m < n ? m : n;
  double f = c * 8.0 * m * k * k;  // the products around the triangular solve
  if (kind == BATCH_POLAR_PB) f += c * 10.0 * 4.0 * n * n * n;  // sign steps
  return f + 1e6;
}

static int pb_plan(int kind, const mak_batch_pullback_item* items, int nitems,
                   const mak_pullback_opts& o, Plan& p) {
  p.owner.assign(nitems, 0);
  p.ws_item.assign(nitems, 0);
  std::vector<int> order(nitems);
  for (int i = 0; i < nitems; i++) {
    order[i] = i;
    Arena meas(nullptr, 0);
    int rc = pb_dispatch(kind, items[i], o, meas, nullptr, 0, 0);
    if (rc != 0) return rc;
    if (kind == BATCH_QR_PB) {
      Arena m2(nullptr, 0);
      rc = rank_dispatch(items[i], o, m2, 0, nullptr);
      if (rc != 0) return rc;
      if (m2.off > meas.off) meas.off = m2.off;
    }
    p.ws_item[i] = meas.off + 512;
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return pb_flops(kind, items[a]) > pb_flops(kind, items[b]);
  });
  double load[kMaxBatchStreams] = {0};
  const int ns = batch_streams();
  for (int s = 0; s < kMaxBatchStreams; s++) p.ws_stream[s] = 0;
  for (int i : order) {
    int best = 0;
    for (int s = 1; s < ns; s++)
      if (load[s] < load[best]) best = s;
    p.owner[i] = best;
    load[best] += pb_flops(kind, items[i]);
    if (p.ws_item[i] > p.ws_stream[best]) p.ws_stream[best] = p.ws_item[i];
  }
  p.total = 0;
  for (int s = 0; s < kMaxBatchStreams; s++) {
    p.off[s] = p.total;
    p.total += align_up(p.ws_stream[s], 256);
  }
  // the ranks of all blocks (QR)
  p.extra_off = p.total;
  p.total += align_up((size_t)(nitems > 0 ? nitems : 1) * sizeof(int), 256);
  return 0;
}

static int pb_validate(int kind, const mak_batch_pullback_item* items, int nitems) {
  if (items == nullptr && nitems > 0) return -1;
  if (nitems < 0) return -2;
  for (int i = 0; i < nitems; i++) {
    const mak_batch_pullback_item& it = items[i];
    const int64_t m = it.m, n = it.n, k = m < n ? m : n;
    if (m < 0 || n < 0 || it.dtype < MAK_F64 || it.dtype > MAK_C32) return -1;
    if (it.dA == nullptr && m * n > 0) return -1;
    if (it.ldda < (m > 1 ? m : 1) || it.ld1 < (m > 1 ? m : 1)) return -1;
    if (kind == BATCH_POLAR_PB && n > m) return -1;
    const int64_t r2 = kind == BATCH_QR_PB ? k : n;  // rows of R / P
    if (it.ld2 < (r2 > 1 ? r2 : 1)) return -1;
    if (it.dF1 != nullptr && it.ldd1 < (m > 1 ? m : 1)) return -1;
    if (it.dF2 != nullptr && it.ldd2 < (r2 > 1 ? r2 : 1)) return -1;
  }
  return 0;
}

static int batched_pb(int kind, const mak_batch_pullback_item* items, int nitems,
                      const mak_pullback_opts* opts, void* work, size_t work_bytes,
                      mak_info* infos, mak_stream_t stream) {
  MAK_TRY(pb_validate(kind, items, nitems));
  mak_pullback_opts o{-1.0, -1.0, MAK_PREC_NATIVE, 0};
  if (opts) o = *opts;
  if (o.precision != MAK_PREC_NATIVE && o.precision != MAK_PREC_MIXED) return -3;
  Plan p;
  MAK_TRY(pb_plan(kind, items, nitems, o, p));
  if (work == nullptr && p.total > 0) return -4;
  if (p.total > work_bytes) return -5;
  if (infos == nullptr && nitems > 0) return -6;
  if (nitems == 0) return 0;
  StreamPool* pp = pool();
  if (pp == nullptr) return MAK_ERR_CUDA;
  StreamPool& sp = *pp;
  cudaStream_t st = (cudaStream_t)stream;
  const int ns = batch_streams();
  int* ranks = (int*)((char*)work + p.extra_off);
  std::vector<int> order(nitems);
  for (int i = 0; i < nitems; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return pb_flops(kind, items[a]) > pb_flops(kind, items[b]);
  });
  auto fork = [&]() -> int {
    MAK_CUDA_TRY(cudaEventRecord(sp.fork, st));
    for (int s = 0; s < ns; s++) MAK_CUDA_TRY(cudaStreamWaitEvent(sp.s[s], sp.fork, 0));
    return 0;
  };
  auto join = [&]() -> int {
    for (int s = 0; s < ns; s++) {
      MAK_CUDA_TRY(cudaEventRecord(sp.join[s], sp.s[s]));
      MAK_CUDA_TRY(cudaStreamWaitEvent(st, sp.join[s], 0));
    }
    return 0;
  };
  std::vector<int> known(nitems, -1);
  int rc_all = 0;
  ThreadSettingsScope settings(false, (int)tuning(TUNE_BATCH_GEMM_CTAS));
  if (kind == BATCH_QR_PB) {
    // every block's rank, then one read of them all
    MAK_TRY(fork());
    for (int i : order) {
      const int s = p.owner[i];
      Arena ar((char*)work + p.off[s], p.ws_stream[s]);
      const int rc = rank_dispatch(items[i], o, ar, sp.s[s], ranks + i);
      if (rc != 0 && rc_all == 0) rc_all = rc;
    }
    MAK_TRY(join());
    if (rc_all != 0) return rc_all;
    MAK_CUDA_TRY(cudaMemcpyAsync(known.data(), ranks, (size_t)nitems * sizeof(int),
                                 cudaMemcpyDeviceToHost, st));
    MAK_CUDA_TRY(cudaStreamSynchronize(st));
  }
  MAK_TRY(fork());
  for (int i : order) {
    const int s = p.owner[i];
    Arena ar((char*)work + p.off[s], p.ws_stream[s]);
    int rc = info_reset(sp.s[s], infos + i);
    if (rc == 0) rc = pb_dispatch(kind, items[i], o, ar, infos + i, sp.s[s], known[i]);
    if (rc != 0 && rc_all == 0) rc_all = rc;
  }
  MAK_TRY(join());
  return rc_all;
}

static int batched_pb_ws(int kind, const mak_batch_pullback_item* items, int nitems,
                         const mak_pullback_opts* opts, size_t* bytes) {
  if (bytes == nullptr) return -4;
  MAK_TRY(pb_validate(kind, items, nitems));
  mak_pullback_opts o{-1.0, -1.0, MAK_PREC_NATIVE, 0};
  if (opts) o = *opts;
  Plan p;
  MAK_TRY(pb_plan(kind, items, nitems, o, p));
  *bytes = p.total + 512;
  return 0;
}

}  // namespace mak

using namespace mak;

extern "C" {

int mak_batched_qr_pullback_workspace(const mak_batch_pullback_item* items, int nitems,
                                      const mak_pullback_opts* opts, size_t* bytes) {
  return batched_pb_ws(BATCH_QR_PB, items, nitems, opts, bytes);
}
int mak_batched_qr_pullback(const mak_batch_pullback_item* items, int nitems,
                            const mak_pullback_opts* opts, void* work, size_t work_bytes,
                            mak_info* infos, mak_stream_t stream) {
  return batched_pb(BATCH_QR_PB, items, nitems, opts, work, work_bytes, infos, stream);
}
int mak_batched_left_polar_pullback_workspace(const mak_batch_pullback_item* items, int nitems,
                                              const mak_pullback_opts* opts, size_t* bytes) {
  return batched_pb_ws(BATCH_POLAR_PB, items, nitems, opts, bytes);
}
int mak_batched_left_polar_pullback(const mak_batch_pullback_item* items, int nitems,
                                    const mak_pullback_opts* opts, void* work, size_t work_bytes,
                                    mak_info* infos, mak_stream_t stream) {
  return batched_pb(BATCH_POLAR_PB, items, nitems, opts, work, work_bytes, infos, stream);
}

int mak_batched_qr_workspace(const mak_batch_item* items, int nitems, const mak_qr_opts* opts,
                             size_t* bytes) {
  return batched_ws(BATCH_QR, items, nitems, opts, bytes);
}
int mak_batched_qr_compact(const mak_batch_item* items, int nitems, const mak_qr_opts* opts,
                           void* work, size_t work_bytes, mak_info* infos, mak_stream_t stream) {
  return batched(BATCH_QR, items, nitems, opts, work, work_bytes, infos, stream);
}
int mak_batched_left_polar_workspace(const mak_batch_item* items, int nitems,
                                     const mak_polar_opts* opts, size_t* bytes) {
  return batched_ws(BATCH_POLAR, items, nitems, opts, bytes);
}
int mak_batched_left_polar(const mak_batch_item* items, int nitems, const mak_polar_opts* opts,
                           void* work, size_t work_bytes, mak_info* infos, mak_stream_t stream) {
  return batched(BATCH_POLAR, items, nitems, opts, work, work_bytes, infos, stream);
}

}  // extern "C"
