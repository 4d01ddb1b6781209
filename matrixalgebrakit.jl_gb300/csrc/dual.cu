// Transposed duals of the QR and polar paths, GB300 native.
//
//   lq_compact! / lq_full!  (reference src/implementations/lq.jl; the
//     LQViaTransposedQR algorithm, src/interface/decompositions.jl:340-353):
//     A = L Q with L lower triangular, positive diagonal, is the conjugate
//     transpose of the positive-diagonal QR of A^H (A^H = Q^H L^H).
//   right_polar!(A, (P, Wh), ::PolarNewton)  (src/implementations/polar.jl:
//     113-125 with right_polar_newton!, polar.jl:168-206): A = P Wh is the
//     conjugate transpose of the left polar decomposition A^H = Wh^H P.  The
//     reference's right Newton iteration on L (from the LQ of A) is the
//     conjugate transpose of the left iteration on R = L^H (the Frobenius
//     scaling and the max-entry stopping test are transpose invariant), so
//     the iterates, iteration count and result agree.
//
// Each entry transposes A into workspace with a tiled kernel, runs the
// existing QR / Newton path on the transpose and transposes the factors into
// the caller's outputs.
#include "internal.h"
#include "util.cuh"

namespace mak {

template <class T>
static int lq_run(cudaStream_t st, int full, int64_t m, int64_t n, const T* A, int64_t lda, T* L,
                  int64_t ldl, T* Q, int64_t ldq, const mak_qr_opts& o, Arena& ar,
                  mak_info* info) {
  const int64_t k = m < n ? m : n;
  const int64_t qr_ = full ? n : k;  // rows of Q (n x n or k x n); columns of L
  T* B = ar.take<T>((size_t)n * m + 1);     // A^H, n x m
  T* QB = ar.take<T>((size_t)n * qr_ + 1);  // Q of A^H, n x qr_
  T* RB = L ? ar.take<T>((size_t)qr_ * m + 1) : nullptr;  // R of A^H, qr_ x m
  size_t inner = 0;
  {
    Arena meas(nullptr, 0);
    qr_run<T>(st, n, m, nullptr, n, nullptr, n, qr_, nullptr, qr_ > 0 ? qr_ : 1, qr_,
              o.positive, o.blocksize, o.precision, meas, nullptr);
    inner = meas.off + 256;
  }
  char* sub = ar.take<char>(inner);
  if (ar.base == nullptr) return 0;
  if (!ar.ok()) return MAK_ERR_WORKSPACE;
  MAK_TRY(ctranspose<T>(st, m, n, A, lda, B, n));
  Arena a2(sub, inner);
  MAK_TRY(qr_run<T>(st, n, m, B, n > 0 ? n : 1, QB, n > 0 ? n : 1, qr_, RB,
                    qr_ > 0 ? qr_ : 1, qr_, o.positive, o.blocksize, o.precision, a2, info));
  MAK_TRY(ctranspose<T>(st, n, qr_, QB, n > 0 ? n : 1, Q, ldq));
  if (L) MAK_TRY(ctranspose<T>(st, qr_, m, RB, qr_ > 0 ? qr_ : 1, L, ldl));
  return 0;
}

template <class T>
static int right_polar_run(cudaStream_t st, int64_t m, int64_t n, const T* A, int64_t lda, T* P,
                           int64_t ldp, T* Wh, int64_t ldwh, int maxiter, double tol,
                           int precision, Arena& ar, mak_info* info) {
  T* B = ar.take<T>((size_t)n * m + 1);   // A^H, n x m
  T* WB = ar.take<T>((size_t)n * m + 1);  // W of A^H, n x m
  size_t inner = 0;
  {
    Arena meas(nullptr, 0);
    polar_newton_run<T>(st, n, m, nullptr, n, nullptr, n, P, ldp, maxiter, tol, precision, meas,
                        nullptr);
    inner = meas.off + 256;
  }
  char* sub = ar.take<char>(inner);
  if (ar.base == nullptr) return 0;
  if (!ar.ok()) return MAK_ERR_WORKSPACE;
  MAK_TRY(ctranspose<T>(st, m, n, A, lda, B, n));
  Arena a2(sub, inner);
  MAK_TRY(polar_newton_run<T>(st, n, m, B, n > 0 ? n : 1, WB, n > 0 ? n : 1, P, ldp, maxiter,
                              tol, precision, a2, info));
  return ctranspose<T>(st, n, m, WB, n > 0 ? n : 1, Wh, ldwh);
}

template <class T>
static int lq_entry(int full, int64_t m, int64_t n, const void* Av, int64_t lda, void* Lv,
                    int64_t ldl, void* Qv, int64_t ldq, const mak_qr_opts* opts, void* work,
                    size_t work_bytes, mak_info* info, mak_stream_t stream) {
  const int64_t k = m < n ? m : n;
  const int64_t qr_ = full ? n : k;
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (Av == nullptr && m * n > 0) return -3;
  if (lda < (m > 1 ? m : 1)) return -4;
  if (Lv && ldl < (m > 1 ? m : 1)) return -6;
  if (Qv == nullptr && qr_ * n > 0) return -7;
  if (ldq < (qr_ > 1 ? qr_ : 1)) return -8;
  mak_qr_opts o{1, 0, MAK_PREC_NATIVE, 0};
  if (opts) o = *opts;
  if (o.blocksize < 0 || o.blocksize > 32) return -9;
  if (o.precision != MAK_PREC_NATIVE && o.precision != MAK_PREC_MIXED) return -9;
  if (info == nullptr) return -12;
  cudaStream_t st = (cudaStream_t)stream;
  {
    Arena meas(nullptr, 0);
    lq_run<T>(st, full, m, n, nullptr, lda, (T*)Lv, ldl, nullptr, ldq, o, meas, nullptr);
    if (meas.off > work_bytes) return -11;
  }
  MAK_TRY(info_reset(st, info));
  Arena ar(work, work_bytes);
  return lq_run<T>(st, full, m, n, (const T*)Av, lda, (T*)Lv, ldl, (T*)Qv, ldq, o, ar, info);
}

template <class T>
static double dual_default_tol() {
  // defaulttol = eps(real T)^(2/3)  (src/common/defaults.jl:10)
  return pow(sizeof(real_t<T>) == 8 ? 2.220446049250313e-16 : 1.1920928955078125e-7, 2.0 / 3.0);
}

template <class T>
static int right_polar_entry(int64_t m, int64_t n, const void* Av, int64_t lda, void* Pv,
                             int64_t ldp, void* Whv, int64_t ldwh, const mak_polar_opts* opts,
                             void* work, size_t work_bytes, mak_info* info, mak_stream_t stream) {
  if (m < 0) return -1;
  if (n < m) return -2;  // n >= m required (polar.jl, check_input of right_polar!)
  if (Av == nullptr && m * n > 0) return -3;
  if (lda < (m > 1 ? m : 1)) return -4;
  if (Pv != nullptr && ldp < (m > 1 ? m : 1)) return -6;
  if (Whv == nullptr && m * n > 0) return -7;
  if (ldwh < (m > 1 ? m : 1)) return -8;
  mak_polar_opts o{10, MAK_PREC_NATIVE, 0.0};
  if (opts) o = *opts;
  if (o.maxiter < 1) return -9;
  if (o.precision != MAK_PREC_NATIVE && o.precision != MAK_PREC_MIXED) return -9;
  const double tol =
      o.tol > 0 ? o.tol : (o.tol < 0 ? -dual_default_tol<T>() : dual_default_tol<T>());
  if (info == nullptr) return -12;
  cudaStream_t st = (cudaStream_t)stream;
  {
    Arena meas(nullptr, 0);
    right_polar_run<T>(st, m, n, nullptr, lda, (T*)Pv, ldp, nullptr, ldwh, o.maxiter, tol,
                       o.precision, meas, nullptr);
    if (meas.off > work_bytes) return -11;
  }
  MAK_TRY(info_reset(st, info));
  Arena ar(work, work_bytes);
  return right_polar_run<T>(st, m, n, (const T*)Av, lda, (T*)Pv, ldp, (T*)Whv, ldwh, o.maxiter,
                            tol, o.precision, ar, info);
}

template <class T>
static size_t lq_ws(int64_t m, int64_t n, int full, const mak_qr_opts& o) {
  Arena meas(nullptr, 0);
  meas.take<mak_info>(1);
  // with L wanted (the larger workspace)
  T dummy;
  lq_run<T>(0, full, m, n, nullptr, m, &dummy, m, nullptr, n, o, meas, nullptr);
  return meas.off + 256;
}
template <class T>
static size_t rpolar_ws(int64_t m, int64_t n, int want_p, const mak_polar_opts& o) {
  Arena meas(nullptr, 0);
  T dummy;
  right_polar_run<T>(0, m, n, nullptr, m, want_p ? &dummy : nullptr, m, nullptr, m,
                     o.maxiter > 0 ? o.maxiter : 10, 1.0, o.precision, meas, nullptr);
  return meas.off + 256;
}

}  // namespace mak

using namespace mak;

extern "C" {

int mak_lq_workspace(int dtype, int64_t m, int64_t n, int full, const mak_qr_opts* opts,
                     size_t* bytes) {
  if (bytes == nullptr) return -6;
  if (m < 0) return -2;
  if (n < 0) return -3;
  mak_qr_opts o{1, 0, MAK_PREC_NATIVE, 0};
  if (opts) o = *opts;
  switch (dtype) {
    case MAK_F64: *bytes = lq_ws<double>(m, n, full, o); break;
    case MAK_C64: *bytes = lq_ws<zcomplex>(m, n, full, o); break;
    case MAK_F32: *bytes = lq_ws<float>(m, n, full, o); break;
    case MAK_C32: *bytes = lq_ws<ccomplex>(m, n, full, o); break;
    default: return -1;
  }
  return 0;
}

int mak_right_polar_workspace(int dtype, int64_t m, int64_t n, int want_p,
                              const mak_polar_opts* opts, size_t* bytes) {
  if (bytes == nullptr) return -6;
  if (m < 0) return -2;
  if (n < m) return -3;
  mak_polar_opts o{10, MAK_PREC_NATIVE, 0.0};
  if (opts) o = *opts;
  switch (dtype) {
    case MAK_F64: *bytes = rpolar_ws<double>(m, n, want_p, o); break;
    case MAK_C64: *bytes = rpolar_ws<zcomplex>(m, n, want_p, o); break;
    case MAK_F32: *bytes = rpolar_ws<float>(m, n, want_p, o); break;
    case MAK_C32: *bytes = rpolar_ws<ccomplex>(m, n, want_p, o); break;
    default: return -1;
  }
  return 0;
}

#define MAK_LQ_ENTRY(NAME, FULL, T, PT)                                                      \
  int NAME(int64_t m, int64_t n, const PT* A, int64_t lda, PT* L, int64_t ldl, PT* Q,        \
           int64_t ldq, const mak_qr_opts* opts, void* work, size_t work_bytes,              \
           mak_info* info, mak_stream_t stream) {                                            \
    return lq_entry<T>(FULL, m, n, A, lda, L, ldl, Q, ldq, opts, work, work_bytes, info,     \
                       stream);                                                              \
  }
MAK_LQ_ENTRY(mak_lq_compact_d, 0, double, double)
MAK_LQ_ENTRY(mak_lq_compact_z, 0, zcomplex, void)
MAK_LQ_ENTRY(mak_lq_compact_s, 0, float, float)
MAK_LQ_ENTRY(mak_lq_compact_c, 0, ccomplex, void)
MAK_LQ_ENTRY(mak_lq_full_d, 1, double, double)
MAK_LQ_ENTRY(mak_lq_full_z, 1, zcomplex, void)
MAK_LQ_ENTRY(mak_lq_full_s, 1, float, float)
MAK_LQ_ENTRY(mak_lq_full_c, 1, ccomplex, void)

#define MAK_RPOLAR_ENTRY(NAME, T, PT)                                                        \
  int NAME(int64_t m, int64_t n, const PT* A, int64_t lda, PT* P, int64_t ldp, PT* Wh,       \
           int64_t ldwh, const mak_polar_opts* opts, void* work, size_t work_bytes,          \
           mak_info* info, mak_stream_t stream) {                                            \
    return right_polar_entry<T>(m, n, A, lda, P, ldp, Wh, ldwh, opts, work, work_bytes,      \
                                info, stream);                                               \
  }
MAK_RPOLAR_ENTRY(mak_right_polar_newton_d, double, double)
MAK_RPOLAR_ENTRY(mak_right_polar_newton_z, zcomplex, void)
MAK_RPOLAR_ENTRY(mak_right_polar_newton_s, float, float)
MAK_RPOLAR_ENTRY(mak_right_polar_newton_c, ccomplex, void)

}  // extern "C"
