// qr_compact! for Float64 without any device allocation at call time.
//
// mak_qr_compact_d takes its scratch from a caller-provided workspace.  Some
// callers cannot provide one: a caller whose device memory is entirely
// owned by its own pool allocator (CUDA.jl's or PyTorch's caching
// allocators) and that must not allocate behind the pool's back, or a
// foreign-language binding that has nowhere to keep a workspace between
// calls.  mak_qr_compact_d_noalloc serves them: its scratch is one fixed
// file-scope device array, so the call itself allocates nothing (no
// cudaMalloc / cudaFree, no allocating library routine).
//
// * The array's size is fixed at MAK_QR_NOALLOC_SCRATCH_BYTES (32 MiB).  When
//   mixed precision is asked for and the split products' planes do not fit,
//   the call runs the native blocking instead (both are FP64-accurate; the
//   precision option chooses speed, not accuracy).  A problem whose native
//   workspace (mak_qr_workspace) exceeds the array as well is rejected with
//   MAK_ERR_WORKSPACE before any work is queued.
// * Set-up, once per device: the first call made while a device is current
//   looks up the array's device address with cudaGetSymbolAddress (this is
//   also when the CUDA runtime loads this file's module and so reserves the
//   array on that device).  That first call must be made before any stream
//   capture begins on that device.
// * Nothing in the array has to start at zero: every call clears the grid
//   barrier words it uses with a stream-ordered memset and writes every
//   other scratch value before reading it.
// * All calls on one device share the array: two calls whose executions
//   overlap (different streams without ordering between them, or different
//   host threads) race on it and produce garbage.  Order such calls on one
//   stream, or with events.
#include <mutex>

#include "internal.h"

namespace mak {

constexpr size_t QR_NOALLOC_SCRATCH_BYTES = (size_t)32 << 20;
static_assert(QR_NOALLOC_SCRATCH_BYTES == MAK_QR_NOALLOC_SCRATCH_BYTES, "header and source agree");

static __device__ __align__(256) unsigned char g_qr_scratch[QR_NOALLOC_SCRATCH_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;

// device address of g_qr_scratch on the current device (looked up once)
static int noalloc_scratch(void** out) {
  static std::mutex mu;
  static void* addr[NOALLOC_MAX_DEVICES] = {};
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return MAK_ERR_CUDA;
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return MAK_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(mu);
  if (addr[dev] == nullptr) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_qr_scratch);
    if (e != cudaSuccess || p == nullptr) return MAK_ERR_CUDA;
    addr[dev] = p;
  }
  *out = addr[dev];
  return 0;
}

}  // namespace mak

using namespace mak;

extern "C" int mak_qr_compact_d_noalloc(int64_t m, int64_t n, double* A, int64_t lda, double* Q,
                                        int64_t ldq, double* R, int64_t ldr,
                                        const mak_qr_opts* opts, mak_info* info,
                                        mak_stream_t stream) {
  if (info == nullptr) return -10;
  size_t need = 0;
  const int rq = mak_qr_workspace(MAK_F64, m, n, 0, opts, &need);
  if (rq != 0) return rq;
  mak_qr_opts o{1, 0, MAK_PREC_NATIVE, 0};
  if (opts) o = *opts;
  if (need > QR_NOALLOC_SCRATCH_BYTES && o.precision == MAK_PREC_MIXED) {
    o.precision = MAK_PREC_NATIVE;  // the split planes do not fit: the native blocking
    if (mak_qr_workspace(MAK_F64, m, n, 0, &o, &need) != 0) return MAK_ERR_WORKSPACE;
  }
  if (need > QR_NOALLOC_SCRATCH_BYTES) return MAK_ERR_WORKSPACE;
  void* scratch = nullptr;
  MAK_TRY(noalloc_scratch(&scratch));
  // the look-ahead path creates its side stream on first use: keep it off
  const bool la = lookahead_enabled();
  set_lookahead(false);
  const int rc = mak_qr_compact_d(m, n, A, lda, Q, ldq, R, ldr, &o, scratch,
                                  QR_NOALLOC_SCRATCH_BYTES, info, stream);
  set_lookahead(la);
  return rc;
}
