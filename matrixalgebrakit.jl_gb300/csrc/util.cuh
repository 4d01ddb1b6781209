// Small memory-bound kernels shared by the polar and pullback paths:
// strided copies, Frobenius / max-abs reductions (deterministic two-level),
// Hermitian projection (smem-tiled so both the (i,j) and (j,i) sides are
// read coalesced -- the reference's GPU kernel walks one side with a stride,
// ext/MatrixAlgebraKitCUDAExt/MatrixAlgebraKitCUDAExt.jl:69-143).
#pragma once
#include "gemm.cuh"

namespace mak {

// B[0:m, 0:n] = alpha * op(A)  (op N or C; C is an out-of-place conjugate transpose)
template <class T>
__global__ void copy_kernel(int64_t m, int64_t n, const T* __restrict__ A, int64_t lda,
                            T* __restrict__ B, int64_t ldb) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int64_t j = blockIdx.y; j < n; j += gridDim.y)
    if (i < m) B[i + j * ldb] = A[i + j * lda];
}
template <class T>
inline int copy_mat(cudaStream_t st, int64_t m, int64_t n, const T* A, int64_t lda, T* B,
                    int64_t ldb) {
  if (m <= 0 || n <= 0) return 0;
  dim3 g((unsigned)ceil_div(m, 256), (unsigned)(n < 65535 ? n : 65535));
  note_launch();
  copy_kernel<T><<<g, 256, 0, st>>>(m, n, A, lda, B, ldb);
  return cudaGetLastError() == cudaSuccess ? 0 : MAK_ERR_CUDA;
}

template <class T>
__global__ void set_identity_kernel(int64_t m, int64_t n, T* B, int64_t ldb) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int64_t j = blockIdx.y; j < n; j += gridDim.y)
    if (i < m) B[i + j * ldb] = (i == j) ? one_<T>() : zero_<T>();
}
template <class T>
inline int set_identity(cudaStream_t st, int64_t m, int64_t n, T* B, int64_t ldb) {
  if (m <= 0 || n <= 0) return 0;
  dim3 g((unsigned)ceil_div(m, 256), (unsigned)(n < 65535 ? n : 65535));
  note_launch();
  set_identity_kernel<T><<<g, 256, 0, st>>>(m, n, B, ldb);
  return cudaGetLastError() == cudaSuccess ? 0 : MAK_ERR_CUDA;
}

// B (n x m) = op(A)^H for A m x n, or B += A^H (ADD): 32 x 32 tiles through
// shared memory so both the read of A and the write of B are coalesced
template <class T, bool ADD>
__global__ void __launch_bounds__(256) ctranspose_kernel(int64_t m, int64_t n,
                                                         const T* __restrict__ A, int64_t lda,
                                                         T* __restrict__ B, int64_t ldb) {
  __shared__ T t[32][33];
  const int64_t i0 = (int64_t)blockIdx.x * 32, j0 = (int64_t)blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  for (int r = ty; r < 32; r += 8) {
    const int64_t i = i0 + tx, j = j0 + r;
    if (i < m && j < n) t[r][tx] = A[i + j * lda];  // t[j - j0][i - i0]
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int64_t j = j0 + tx, i = i0 + r;  // B[j, i] = conj(A[i, j])
    if (i < m && j < n) {
      const T v = conj_(t[tx][r]);
      if (ADD) B[j + i * ldb] += v;
      else B[j + i * ldb] = v;
    }
  }
}
template <class T>
inline int ctranspose(cudaStream_t st, int64_t m, int64_t n, const T* A, int64_t lda, T* B,
                      int64_t ldb, bool add = false) {
  if (m <= 0 || n <= 0) return 0;
  if (ceil_div(n, 32) > 65535) return MAK_ERR_UNSUPPORTED;
  dim3 g((unsigned)ceil_div(m, 32), (unsigned)ceil_div(n, 32));
  note_launch();
  if (add) ctranspose_kernel<T, true><<<g, 256, 0, st>>>(m, n, A, lda, B, ldb);
  else ctranspose_kernel<T, false><<<g, 256, 0, st>>>(m, n, A, lda, B, ldb);
  return cudaGetLastError() == cudaSuccess ? 0 : MAK_ERR_CUDA;
}

// ---- reductions -------------------------------------------------------------
// Partial results per CTA, then one CTA folds them in a fixed order.
constexpr int RED_CTAS = 304;

// kind 0: sum |a|^2 (Frobenius^2), kind 1: max |a|
template <class T>
__global__ void __launch_bounds__(256) reduce_partial_kernel(int64_t m, int64_t n, const T* A,
                                                             int64_t lda, int kind,
                                                             real_t<T>* part) {
  using R = real_t<T>;
  __shared__ R sh[32];
  const int64_t total = m * n;
  R acc = R(0);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e % m, j = e / m;
    T v = A[i + j * lda];
    if (kind == 0) acc += abs2_(v);
    else acc = fmax(acc, abs_(v));
  }
  R r = (kind == 0) ? block_sum(acc, sh) : block_max(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = r;
}
template <class R>
__global__ void __launch_bounds__(256) reduce_final_kernel(int np, const R* part, int kind,
                                                           R* out) {
  __shared__ R sh[32];
  R acc = R(0);
  for (int q = threadIdx.x; q < np; q += blockDim.x)
    acc = (kind == 0) ? acc + part[q] : fmax(acc, part[q]);
  R r = (kind == 0) ? block_sum(acc, sh) : block_max(acc, sh);
  if (threadIdx.x == 0) *out = r;
}
// *out = ||A||_F^2 (kind 0) or max|A| (kind 1); `part` holds RED_CTAS reals
template <class T>
inline int reduce_mat(cudaStream_t st, int64_t m, int64_t n, const T* A, int64_t lda, int kind,
                      real_t<T>* part, real_t<T>* out) {
  int64_t total = m * n;
  int g = (int)(total <= 0 ? 1 : ceil_div(total, 256));
  if (g > RED_CTAS) g = RED_CTAS;
  note_launch();
  reduce_partial_kernel<T><<<g, 256, 0, st>>>(m > 0 ? m : 1, total > 0 ? n : 0, A, lda, kind,
                                              part);
  note_launch();
  reduce_final_kernel<real_t<T>><<<1, 256, 0, st>>>(g, part, kind, out);
  return cudaGetLastError() == cudaSuccess ? 0 : MAK_ERR_CUDA;
}

// ---- Hermitian projection, in place: A <- (A + A^H)/2, real diagonal --------
// (reference project_hermitian!, src/implementations/projections.jl:61-108)
// Each CTA owns the tile pair (I,J), (J,I) with I <= J.
template <class T>
__global__ void __launch_bounds__(256) herm_project_kernel(int64_t n, T* A, int64_t lda) {
  __shared__ T t1[32][33];
  __shared__ T t2[32][33];
  const int64_t bi = blockIdx.x, bj = blockIdx.y;
  if (bi > bj) return;
  const int64_t i0 = bi * 32, j0 = bj * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  for (int r = ty; r < 32; r += 8) {
    int64_t i = i0 + tx, j = j0 + r;
    t1[r][tx] = (i < n && j < n) ? A[i + j * lda] : zero_<T>();     // t1[c][r] = A[i0+r', j0+c]
    int64_t i2 = j0 + tx, j2 = i0 + r;
    t2[r][tx] = (i2 < n && j2 < n) ? A[i2 + j2 * lda] : zero_<T>();  // t2[c][r] = A[j0+r', i0+c]
  }
  __syncthreads();
  const real_t<T> half = real_t<T>(0.5);
  for (int r = ty; r < 32; r += 8) {
    // element (i0+tx, j0+r): (A[i,j] + conj(A[j,i]))/2, A[j,i] = t2[tx][r]
    int64_t i = i0 + tx, j = j0 + r;
    if (i < n && j < n) {
      T v = half * (t1[r][tx] + conj_(t2[tx][r]));
      if (i == j) v = make_scalar<T>(re_(v), 0);
      A[i + j * lda] = v;
    }
    int64_t i2 = j0 + tx, j2 = i0 + r;
    if (bi != bj && i2 < n && j2 < n) {
      T v = half * (t2[r][tx] + conj_(t1[tx][r]));
      A[i2 + j2 * lda] = v;
    }
  }
}
template <class T>
inline int herm_project(cudaStream_t st, int64_t n, T* A, int64_t lda) {
  if (n <= 0) return 0;
  dim3 g((unsigned)ceil_div(n, 32), (unsigned)ceil_div(n, 32));
  note_launch();
  herm_project_kernel<T><<<g, 256, 0, st>>>(n, A, lda);
  return cudaGetLastError() == cudaSuccess ? 0 : MAK_ERR_CUDA;
}

}  // namespace mak
