// Native-precision tiled GEMM on the SIMT pipes (FP64 DFMA, FP32 FFMA,
// complex as 4 real FMAs), with structured operands.
//
//   C = alpha * op(A) * op(B) + beta * C
//
// op(X) in {N, T, C}; each operand may additionally be read through a
// structure mask of its *stored* matrix: unit-lower-trapezoidal (Householder
// V: implicit 1 on the diagonal, 0 above), upper or lower triangular.  This
// lets the larfb / orgqr / pullback products read V and R straight out of the
// packed QR storage without materialising copies.
//
// On GB300 FP64 runs at ~1 TFLOP/s for the whole chip (measured: DFMA and
// DMMA alike), i.e. ~3.3 flop/clk/SM, so a plain 64x64x16 smem tile is already
// issue-bound on the FP64 pipe; the tensor-core path is the split-precision
// GEMM in ozaki.cuh.
#pragma once
#include "mak_common.cuh"

namespace mak {

enum Op { OP_N = 0, OP_T = 1, OP_C = 2 };
enum Mask { MASK_FULL = 0, MASK_UNIT_LOWER = 1, MASK_UPPER = 2, MASK_LOWER = 3 };

template <class T>
struct Operand {
  const T* p;
  int64_t ld;
  int op;
  int mask;
};
template <class T>
inline Operand<T> opnd(const T* p, int64_t ld, int op = OP_N, int mask = MASK_FULL) {
  return Operand<T>{p, ld, op, mask};
}

// element (i, k) of op(X); (r, c) is the position in the stored matrix
template <class T>
__device__ __forceinline__ T load_op(const Operand<T>& X, int64_t i, int64_t k) {
  int64_t r = (X.op == OP_N) ? i : k;
  int64_t c = (X.op == OP_N) ? k : i;
  switch (X.mask) {
    case MASK_UNIT_LOWER:
      if (r < c) return zero_<T>();
      if (r == c) return one_<T>();
      break;
    case MASK_UPPER:
      if (r > c) return zero_<T>();
      break;
    case MASK_LOWER:
      if (r < c) return zero_<T>();
      break;
    default:
      break;
  }
  T v = X.p[r + c * X.ld];
  return X.op == OP_C ? conj_(v) : v;
}

template <class T>
__device__ __forceinline__ bool is_zero_(T v) { return v == zero_<T>(); }

template <class T, int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
gemm_kernel(int M, int N, int K, T alpha, Operand<T> A, Operand<T> B, T beta, T* C,
            int64_t ldc, int kchunk, int64_t split_stride, const int* skip) {
  if (skipped(skip)) return;
  constexpr int RX = BM / TM;  // threads along rows
  constexpr int RY = BN / TN;  // threads along columns
  constexpr int NT = RX * RY;
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int64_t m0 = (int64_t)blockIdx.x * BM;
  const int64_t n0 = (int64_t)blockIdx.y * BN;
  const int kbeg = blockIdx.z * kchunk;
  const int kend = min(K, kbeg + kchunk);
  C += blockIdx.z * split_stride;
  const int tid = threadIdx.x;
  const int tx = tid % RX, ty = tid / RX;
  T acc[TM][TN];
#pragma unroll
  for (int r = 0; r < TM; r++)
#pragma unroll
    for (int c = 0; c < TN; c++) acc[r][c] = zero_<T>();

  for (int k0 = kbeg; k0 < kend; k0 += BK) {
    for (int e = tid; e < BM * BK; e += NT) {
      int ii, kk;
      if (A.op == OP_N) { ii = e % BM; kk = e / BM; } else { kk = e % BK; ii = e / BK; }
      int64_t gi = m0 + ii;
      int gk = k0 + kk;
      As[kk][ii] = (gi < M && gk < kend) ? load_op(A, gi, gk) : zero_<T>();
    }
    for (int e = tid; e < BK * BN; e += NT) {
      int kk, jj;
      if (B.op == OP_N) { kk = e % BK; jj = e / BK; } else { jj = e % BN; kk = e / BN; }
      int64_t gj = n0 + jj;
      int gk = k0 + kk;
      Bs[kk][jj] = (gj < N && gk < kend) ? load_op(B, gk, gj) : zero_<T>();
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < BK; kk++) {
      T a[TM], b[TN];
#pragma unroll
      for (int r = 0; r < TM; r++) a[r] = As[kk][tx + r * RX];
#pragma unroll
      for (int c = 0; c < TN; c++) b[c] = Bs[kk][ty + c * RY];
#pragma unroll
      for (int r = 0; r < TM; r++)
#pragma unroll
        for (int c = 0; c < TN; c++) acc[r][c] = fma_(a[r], b[c], acc[r][c]);
    }
    __syncthreads();
  }
  const bool use_beta = !is_zero_(beta);
#pragma unroll
  for (int c = 0; c < TN; c++) {
    int64_t j = n0 + ty + c * RY;
    if (j >= N) continue;
#pragma unroll
    for (int r = 0; r < TM; r++) {
      int64_t i = m0 + tx + r * RX;
      if (i >= M) continue;
      T v = alpha * acc[r][c];
      if (use_beta) v = fma_(beta, C[i + j * ldc], v);
      C[i + j * ldc] = v;
    }
  }
}

template <class T>
__global__ void scale_kernel(int M, int N, T beta, T* C, int64_t ldc) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t j = blockIdx.y;
  if (i < M && j < N) C[i + j * ldc] = is_zero_(beta) ? zero_<T>() : beta * C[i + j * ldc];
}

// Host launcher.  `splits` > 1 partitions K; split s writes its partial
// product (beta ignored, treated as 0) to C + s * split_stride.
template <class T>
int gemm(cudaStream_t st, int64_t M, int64_t N, int64_t K, T alpha, Operand<T> A,
         Operand<T> B, T beta, T* C, int64_t ldc, int splits = 1, int64_t split_stride = 0,
         int* used_splits = nullptr) {
  if (used_splits) *used_splits = 1;
  if (M <= 0 || N <= 0) return 0;
  if (K <= 0) {
    dim3 g((unsigned)ceil_div(M, 256), (unsigned)N);
    note_launch();
    scale_kernel<T><<<g, 256, 0, st>>>((int)M, (int)N, beta, C, ldc);
    return cudaGetLastError() == cudaSuccess ? 0 : MAK_ERR_CUDA;
  }
  if (splits < 1) splits = 1;
  constexpr int BK = 16;
  int kchunk = (int)ceil_div(ceil_div(K, splits), BK) * BK;
  splits = (int)ceil_div(K, kchunk);
  if (used_splits) *used_splits = splits;
  if (splits > 1) beta = zero_<T>();
  ProfScope prof(st, PROF_GEMM_NATIVE, (traits<T>::cpx ? 8.0 : 2.0) * M * N * K);
  if (M <= 32) {
    dim3 g((unsigned)ceil_div(M, 32), (unsigned)ceil_div(N, 64), (unsigned)splits);
    note_launch();
    gemm_kernel<T, 32, 64, BK, 2, 4><<<g, 256, 0, st>>>((int)M, (int)N, (int)K, alpha, A, B,
                                                         beta, C, ldc, kchunk, split_stride,
                                                         skip_flag());
  } else {
    dim3 g((unsigned)ceil_div(M, 64), (unsigned)ceil_div(N, 64), (unsigned)splits);
    note_launch();
    gemm_kernel<T, 64, 64, BK, 4, 4><<<g, 256, 0, st>>>((int)M, (int)N, (int)K, alpha, A, B,
                                                         beta, C, ldc, kchunk, split_stride,
                                                         skip_flag());
  }
  return cudaGetLastError() == cudaSuccess ? 0 : MAK_ERR_CUDA;
}

// number of K-splits that fills the GPU for an output of M x N
inline int pick_splits(int64_t M, int64_t N, int64_t K, int sms) {
  int64_t tiles = ceil_div(M, M <= 32 ? 32 : 64) * ceil_div(N, 64);
  int64_t want = 2LL * sms;
  if (tiles >= want) return 1;
  int64_t s = ceil_div(want, tiles);
  int64_t maxs = ceil_div(K, 64);  // keep >= 64 of K per split
  if (s > maxs) s = maxs;
  if (s < 1) s = 1;
  if (s > 64) s = 64;
  return (int)s;
}

}  // namespace mak
