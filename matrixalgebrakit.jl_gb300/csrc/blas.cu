// GEMM dispatch (native SIMT or split-precision tensor core) and its C entry
// points.  The library's factorizations call gemm_prec for every large
// product; mak_gemm_* expose the same dispatch to callers and tests.
#include "gemm.cuh"
#include "internal.h"

#include <cstdlib>
#include <mutex>

namespace mak {

double split_min_mnk() { return tuning(TUNE_SPLIT_MIN_MNK); }

// C = alpha * sum_s part[s] + beta * C  (fixed summation order)
template <class T>
__global__ void splitk_fold_kernel(int64_t M, int64_t N, int splits, const T* part, T alpha,
                                   T beta, T* C, int64_t ldc, const int* skip) {
  if (skipped(skip)) return;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= M * N) return;
  T v = zero_<T>();
  for (int s = 0; s < splits; s++) v += part[s * M * N + e];
  const int64_t i = e % M, j = e / M;
  T out = alpha * v;
  if (!is_zero_(beta)) out = fma_(beta, C[i + j * ldc], out);
  C[i + j * ldc] = out;
}

// native product: split K across CTAs when the output alone cannot fill the GPU
template <class T>
static int gemm_native(cudaStream_t st, int64_t M, int64_t N, int64_t K, T alpha, Operand<T> A,
                       Operand<T> B, T beta, T* C, int64_t ldc, Arena& ar) {
  const int splits = (M > 0 && N > 0 && K > 0) ? pick_splits(M, N, K, num_sms()) : 1;
  if (ar.base == nullptr) {
    // measuring: a bound valid for every smaller output too (pick_splits
    // keeps splits * tiles <= 4 * SMs), since the split count grows as the
    // output shrinks while call sites measure at their largest shape
    if (K > 64) {  // pick_splits keeps >= 64 of K per split
      const size_t bound = (size_t)4 * num_sms() * 64 * 64;
      const size_t cap = (size_t)64 * (size_t)(M > 0 ? M : 1) * (size_t)(N > 0 ? N : 1);
      ar.take<T>(bound < cap ? bound : cap);
    }
    return 0;
  }
  if (splits <= 1) return gemm<T>(st, M, N, K, alpha, A, B, beta, C, ldc);
  T* part = ar.take<T>((size_t)splits * M * N);
  if (ar.base == nullptr) return 0;
  if (!ar.ok()) return MAK_ERR_WORKSPACE;
  int used = 1;
  MAK_TRY(gemm<T>(st, M, N, K, one_<T>(), A, B, zero_<T>(), part, M, splits, M * N, &used));
  note_launch();
  splitk_fold_kernel<T><<<(unsigned)ceil_div(M * N, 256), 256, 0, st>>>(M, N, used, part, alpha,
                                                                       beta, C, ldc, skip_flag());
  return cudaGetLastError() == cudaSuccess ? 0 : MAK_ERR_CUDA;
}

// Inside the factorizations MAK_PREC_MIXED takes the split product only
// when the product is large enough to repay its fixed cost (exponent pass,
// plane split, TMEM set-up: a few tens of microseconds); smaller products
// stay native.  PREC_SPLIT_ALWAYS (the C-ABI GEMM) takes it at every size.
// A measuring pass (ar.base == nullptr) reserves the larger of both paths'
// workspace, because call sites measure at their largest shape.
template <class T>
int gemm_prec(cudaStream_t st, int precision, int64_t M, int64_t N, int64_t K, T alpha,
              Operand<T> A, Operand<T> B, T beta, T* C, int64_t ldc, Arena& ar, int* status,
              int max_ctas) {
  if constexpr (sizeof(real_t<T>) == 8) {
    const bool can_split = (precision == MAK_PREC_MIXED || precision == PREC_SPLIT_ALWAYS) &&
                           im_(alpha) == 0 && im_(beta) == 0 && K >= 16;
    if (can_split) {
      if (ar.base == nullptr) {
        Arena a1 = ar, a2 = ar;
        oz_gemm<T>(st, M, N, K, alpha, A, B, beta, C, ldc, a1, status);
        gemm_native<T>(st, M, N, K, alpha, A, B, beta, C, ldc, a2);
        ar.off = a1.off > a2.off ? a1.off : a2.off;
        return 0;
      }
      const double work = (traits<T>::cpx ? 4.0 : 1.0) * (double)M * (double)N * (double)K;
      if (precision == PREC_SPLIT_ALWAYS || work >= split_min_mnk())
        return oz_gemm<T>(st, M, N, K, alpha, A, B, beta, C, ldc, ar, status, max_ctas);
    }
  }
  return gemm_native<T>(st, M, N, K, alpha, A, B, beta, C, ldc, ar);
}

#define MAK_INST_GP(T)                                                                        \
  template int gemm_prec<T>(cudaStream_t, int, int64_t, int64_t, int64_t, T, Operand<T>,      \
                            Operand<T>, T, T*, int64_t, Arena&, int*, int);
MAK_INST_GP(double)
MAK_INST_GP(float)
MAK_INST_GP(zcomplex)
MAK_INST_GP(ccomplex)

template <class T>
static int gemm_entry(int opA, int opB, int64_t m, int64_t n, int64_t k, T alpha, const T* A,
                      int64_t lda, const T* B, int64_t ldb, T beta, T* C, int64_t ldc,
                      int precision, void* work, size_t work_bytes, mak_info* info,
                      mak_stream_t stream) {
  if (opA < 0 || opA > 2) return -1;
  if (opB < 0 || opB > 2) return -2;
  if (m < 0) return -3;
  if (n < 0) return -4;
  if (k < 0) return -5;
  const int64_t ar_rows = (opA == OP_N) ? m : k;
  const int64_t br_rows = (opB == OP_N) ? k : n;
  if (A == nullptr && m * k > 0) return -7;
  if (lda < (ar_rows > 1 ? ar_rows : 1)) return -8;
  if (B == nullptr && k * n > 0) return -9;
  if (ldb < (br_rows > 1 ? br_rows : 1)) return -10;
  if (C == nullptr && m * n > 0) return -12;
  if (ldc < (m > 1 ? m : 1)) return -13;
  if (precision != MAK_PREC_NATIVE && precision != MAK_PREC_MIXED) return -14;
  if (info == nullptr) return -17;
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == MAK_PREC_MIXED) precision = PREC_SPLIT_ALWAYS;  // the caller chose
  Operand<T> a = opnd<T>(A, lda, opA), b = opnd<T>(B, ldb, opB);
  {
    Arena meas(nullptr, 0);
    gemm_prec<T>(st, precision, m, n, k, alpha, a, b, beta, nullptr, ldc, meas, nullptr);
    if (meas.off > work_bytes) return -16;
  }
  MAK_TRY(info_reset(st, info));
  Arena ar(work, work_bytes);
  return gemm_prec<T>(st, precision, m, n, k, alpha, a, b, beta, C, ldc, ar, &info->status);
}

}  // namespace mak

using namespace mak;

extern "C" {

int mak_gemm_workspace(int dtype, int opA, int opB, int64_t m, int64_t n, int64_t k,
                       int precision, size_t* bytes) {
  if (bytes == nullptr) return -8;
  Arena meas(nullptr, 0);
  switch (dtype) {
    case MAK_F64: gemm_prec<double>(0, precision, m, n, k, 1.0, opnd<double>(nullptr, 1, opA), opnd<double>(nullptr, 1, opB), 0.0, nullptr, 1, meas, nullptr); break;
    case MAK_C64: gemm_prec<zcomplex>(0, precision, m, n, k, zcomplex(1.0), opnd<zcomplex>(nullptr, 1, opA), opnd<zcomplex>(nullptr, 1, opB), zcomplex(0.0), nullptr, 1, meas, nullptr); break;
    case MAK_F32: case MAK_C32: break;
    default: return -1;
  }
  *bytes = meas.off + 256;
  return 0;
}

int mak_gemm_d(int opA, int opB, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
               int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
               int precision, void* work, size_t work_bytes, mak_info* info,
               mak_stream_t stream) {
  return gemm_entry<double>(opA, opB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, precision,
                            work, work_bytes, info, stream);
}

int mak_gemm_z(int opA, int opB, int64_t m, int64_t n, int64_t k, const double* alpha,
               const void* A, int64_t lda, const void* B, int64_t ldb, const double* beta,
               void* C, int64_t ldc, int precision, void* work, size_t work_bytes,
               mak_info* info, mak_stream_t stream) {
  if (alpha == nullptr) return -6;
  if (beta == nullptr) return -11;
  return gemm_entry<zcomplex>(opA, opB, m, n, k, zcomplex(alpha[0], alpha[1]),
                              (const zcomplex*)A, lda, (const zcomplex*)B, ldb,
                              zcomplex(beta[0], beta[1]), (zcomplex*)C, ldc, precision, work,
                              work_bytes, info, stream);
}

}  // extern "C"
