// Reverse-mode rules of the QR and left polar decompositions, GB300 native.
//
// qr_pullback (reference src/pullbacks/qr.jl:1-120):
//   p   = last j with |R_jj| >= rank_atol   (rank_atol = eps(max|R|)^(3/4))
//   gauge check of the cotangents (qr.jl:4-53), reported in info->gauge
//   dQ1 -= Q1 (dR12 R12^H);  dA2 += Q1 dR12                       (n > p)
//   M    = triu(dR11) R11^H - Q1^H dQ1;  M <- copyltu(M), real diagonal
//   dQ1 += Q1 M;             dA1 += dQ1 R11^{-H}
//   The triangular solve uses the explicit inverse of R11 from the
//   Gauss-Jordan kernel (no pivot exchanges occur on a triangular matrix).
//
// left_polar_pullback (reference src/pullbacks/polar.jl:7-29):
//   dP <- herm(dP);  M = W^H dW - dP P;  solve P C + C P = M - M^H;
//   C += dP;  dA += W C;  dA += (I - W W^H) dW P^{-1}
//   The Sylvester equation is solved on the device (the reference's CUDA
//   extension copies P to the host for LAPACK trsyl,
//   ext/MatrixAlgebraKitCUDAExt/MatrixAlgebraKitCUDAExt.jl:193-198) by the
//   Newton iteration for the matrix sign function of H = [[P, -B], [0, -P]]:
//   sign(H) = [[I, -2X], [0, -I]] with P X + X P = B.  With
//   H_k = [[A_k, C_k], [0, -A_k]] the iteration decouples into
//     A_{k+1} = (mu A_k + A_k^{-1}/mu)/2,
//     C_{k+1} = (mu C_k + A_k^{-1} C_k A_k^{-1}/mu)/2,
//   A_0 = P, C_0 = -B, mu = sqrt(||A_k^{-1}||_F / ||A_k||_F); X = -C_inf/2.
//   Only GEMMs and the Gauss-Jordan inverse are needed (no eigensolver).
#include "gemm.cuh"
#include "internal.h"
#include "util.cuh"

namespace mak {

// ---------------------------------------------------------------- helpers --
// eps(x)^(3/4) of Julia (`eps(x)` = spacing of floats at x; at 0 and in the
// subnormal range that spacing is the smallest subnormal, so the tolerance
// stays positive and an all-zero R has rank 0, as in the reference)
template <class R>
__device__ __forceinline__ R eps34(R x) {
  const int mant = sizeof(R) == 8 ? 52 : 23;
  const R tiny = ldexp(R(1), sizeof(R) == 8 ? -1074 : -149);  // smallest subnormal
  R sp = tiny;
  if (x > R(0)) {
    int e;
    frexp(x, &e);  // x = f 2^e, f in [0.5, 1)
    const R s = ldexp(R(1), e - 1 - mant);
    sp = s > tiny ? s : tiny;
  }
  return pow(sp, R(0.75));
}

// p = 1 + last j < k with |R_jj| >= atol (atol < 0: eps(maxR)^(3/4)); 0 if none
template <class T>
__global__ void qr_rank_kernel(int k, const T* R, int64_t ldr, const real_t<T>* maxR,
                               double atol_in, int* p_out, real_t<T>* atol_out) {
  using Rr = real_t<T>;
  __shared__ int best[32];
  const Rr atol = atol_in >= 0 ? (Rr)atol_in : eps34(*maxR);
  int b = 0;
  for (int j = threadIdx.x; j < k; j += blockDim.x)
    if (abs_(R[j + (int64_t)j * ldr]) >= atol) b = j + 1 > b ? j + 1 : b;
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) {
    int o = __shfl_xor_sync(0xffffffffu, b, m);
    b = o > b ? o : b;
  }
  if ((threadIdx.x & 31) == 0) best[threadIdx.x >> 5] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    int r = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) r = best[w] > r ? best[w] : r;
    *p_out = r;
    if (atol_out) *atol_out = atol;
  }
}

// max over the upper triangle (incl. diagonal) of X (rows x cols) -> *out (max-combine)
template <class T>
__global__ void max_upper_kernel(int rows, int cols, const T* X, int64_t ldx, real_t<T>* out) {
  using Rr = real_t<T>;
  __shared__ Rr sh[32];
  Rr mx = Rr(0);
  const int64_t total = (int64_t)rows * cols;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % rows), j = (int)(e / rows);
    if (i <= j) mx = fmax(mx, abs_(X[i + (int64_t)j * ldx]));
  }
  mx = block_max(mx, sh);
  if (threadIdx.x == 0) {
    // non-negative reals compare like their bit patterns
    if (sizeof(Rr) == 8)
      atomicMax((unsigned long long*)out, (unsigned long long)__double_as_longlong((double)mx));
    else
      atomicMax((unsigned int*)out, __float_as_uint((float)mx));
  }
}

// M <- copyltu(M): lower triangle = conj(upper), real diagonal (qr.jl:108-112)
template <class T>
__global__ void copyltu_kernel(int p, T* M, int64_t ldm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= p || j >= p) return;
  if (i > j) M[i + (int64_t)j * ldm] = conj_(M[j + (int64_t)i * ldm]);
  else if (i == j) M[i + (int64_t)i * ldm] = make_scalar<T>(re_(M[i + (int64_t)i * ldm]), 0);
}

// B = s (M - M^H)   (n x n, out of place)
template <class T>
__global__ void antiherm_kernel(int n, const T* M, int64_t ldm, real_t<T> s, T* B, int64_t ldb) {
  __shared__ T t[32][33];
  const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int r = ty; r < 32; r += 8) {
    const int i = j0 + tx, j = i0 + r;  // load M[j0+tx, i0+r] -> t[r][tx]
    t[r][tx] = (i < n && j < n) ? M[i + (int64_t)j * ldm] : zero_<T>();
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + tx, j = j0 + r;
    if (i < n && j < n) B[i + (int64_t)j * ldb] = s * (M[i + (int64_t)j * ldm] - conj_(t[tx][r]));
  }
}

// Y[:, c] = X[:, iperm[c]]  (explicit inverse from the Gauss-Jordan output)
template <class T>
__global__ void gather_cols_kernel(int n, const T* X, int64_t ldx, const int* iperm, T* Y,
                                   int64_t ldy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (i < n && c < n) Y[i + (int64_t)c * ldy] = X[i + (int64_t)iperm[c] * ldx];
}

// sign-iteration update, mu = (||Ai||^2/||A||^2)^(1/4):
//   A <- (mu A + Ai/mu)/2,  C <- (mu C + Tm/mu)/2,  *dnorm += |A_new - A_old|^2 (partial)
template <class T>
__global__ void sign_update_kernel(int64_t nn, T* A, const T* Ai, T* Cm, const T* Tm,
                                   const real_t<T>* nrm2, real_t<T>* dpart, const int* skip) {
  using Rr = real_t<T>;
  if (skipped(skip)) return;
  __shared__ Rr sh[32];
  const Rr mu = sqrt(sqrt(nrm2[1] / nrm2[0]));
  const Rr imu = Rr(1) / mu;
  Rr acc = Rr(0);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x) {
    const T a = A[e];
    const T an = Rr(0.5) * (mu * a + imu * Ai[e]);
    A[e] = an;
    acc += abs2_(an - a);
    Cm[e] = Rr(0.5) * (mu * Cm[e] + imu * Tm[e]);
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) dpart[blockIdx.x] = acc;
}

// Device stop of the sign iteration without host synchronization: w[0] is
// the stop flag the later iterations' kernels read on entry, w[1] counts the
// iterations taken (NaN stops, as the host-checked loop does).
template <class R>
__global__ void sign_stop_kernel(const R* dnorm2, R tol, int* w) {
  if (w[0]) return;
  w[1] += 1;
  if (!(sqrt(*dnorm2) > tol)) w[0] = 1;
}
__global__ void info_sign_fixed_kernel(mak_info* info, const int* w) {
  info->iterations = w[1];
  info->converged = w[0];
}

template <class R>
__global__ void eps34_kernel(const R* x, R* out) {
  *out = eps34(*x);
}

// Y[0:m, 0:n] += X (both strided)
template <class T>
__global__ void add_strided_kernel(int64_t m, int64_t n, const T* X, int64_t ldx, T* Y,
                                   int64_t ldy) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int64_t j = blockIdx.y; j < n; j += gridDim.y)
    if (i < m) Y[i + j * ldy] += X[i + j * ldx];
}

template <class T>
__global__ void scale_copy_kernel(int64_t nn, const T* X, real_t<T> s, T* Y) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < nn) Y[e] = s * X[e];
}
template <class T>
__global__ void add_kernel(int64_t nn, const T* X, T* Y) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < nn) Y[e] += X[e];
}

template <class T>
__global__ void info_pullback_kernel(mak_info* info, int p, int iters, const real_t<T>* gauge,
                                     const real_t<T>* gauge_atol) {
  info->rank = p;
  info->iterations = iters;
  info->gauge = gauge ? (double)*gauge : 0.0;
  info->gauge_atol = gauge_atol ? (double)*gauge_atol : 0.0;
}

// -------------------------------------------------------------- QR pullback --
// known_p >= 0: the numerical rank was computed beforehand (qr_rank_run,
// e.g. for a whole batch at once) and no host synchronization is needed.
template <class T>
int qr_pullback_run(cudaStream_t st, int64_t m, int64_t n, int full, T* dA, int64_t ldda,
                    const T* Q, int64_t ldq, const T* R, int64_t ldr, const T* dQ, int64_t lddq,
                    const T* dR, int64_t lddr, double rank_atol, double gauge_atol, int precision,
                    Arena& ar, mak_info* info, int known_p) {
  using Rr = real_t<T>;
  const int64_t k = m < n ? m : n;
  const int64_t qc = full ? m : k;
  Rr* scal = ar.take<Rr>(RED_CTAS + 16);  // reductions + scalars
  int* pdev = ar.take<int>(4);
  T* dQ1 = ar.take<T>((size_t)m * (k > 0 ? k : 1));
  T* X = ar.take<T>((size_t)(k > 0 ? k : 1) * (k > 0 ? k : 1));
  T* Mm = ar.take<T>((size_t)(k > 0 ? k : 1) * (k > 0 ? k : 1));
  T* Rinv = ar.take<T>((size_t)(k > 0 ? k : 1) * (k > 0 ? k : 1));
  int* iperm = ar.take<int>(k + 1);
  T* Q1dQ3 = (full && qc > k) ? ar.take<T>((size_t)k * (qc - k)) : nullptr;
  T* dQ3 = (full && qc > k) ? ar.take<T>((size_t)m * (qc - k)) : nullptr;
  size_t gj_ws = 0, oz_ws = 0;
  {
    Arena meas(nullptr, 0);
    gje_inverse<T>(st, k, nullptr, k, nullptr, precision, meas, nullptr);
    gj_ws = meas.off + 256;
    const int64_t shapes[4][3] = {{k, k, n}, {m, n, k}, {k, k, m}, {m, k, k}};
    for (auto& sh : shapes) {
      Arena m2(nullptr, 0);
      gemm_prec<T>(st, precision, sh[0], sh[1], sh[2], one_<T>(), opnd<T>(nullptr, 1),
                   opnd<T>(nullptr, 1), zero_<T>(), nullptr, 1, m2, nullptr);
      if (m2.off + 256 > oz_ws) oz_ws = m2.off + 256;
    }
  }
  const size_t tail_bytes = gj_ws > oz_ws ? gj_ws : oz_ws;
  char* tail = ar.take<char>(tail_bytes);
  if (ar.base == nullptr) return 0;
  if (!ar.ok()) return MAK_ERR_WORKSPACE;
  int* status = &info->status;
  Rr* red = scal;
  Rr* maxR = scal + RED_CTAS;
  Rr* gauge = scal + RED_CTAS + 1;
  Rr* gatol = scal + RED_CTAS + 2;
  Rr* ratol = scal + RED_CTAS + 3;
  Rr* tmp = scal + RED_CTAS + 4;
  auto G = [&](int64_t M_, int64_t N_, int64_t K_, T alpha, Operand<T> a, Operand<T> b, T beta,
               T* C_, int64_t ldc) -> int {
    Arena oz(tail, tail_bytes);
    return gemm_prec<T>(st, precision, M_, N_, K_, alpha, a, b, beta, C_, ldc, oz, status);
  };

  // rank
  MAK_CUDA_TRY(cudaMemsetAsync(scal + RED_CTAS, 0, 16 * sizeof(Rr), st));
  MAK_TRY(reduce_mat<T>(st, k, n, R, ldr, 1, red, maxR));
  note_launch();
  qr_rank_kernel<T><<<1, 256, 0, st>>>((int)k, R, ldr, maxR, rank_atol, pdev, ratol);
  MAK_CUDA_TRY(cudaGetLastError());
  int p = known_p;
  if (p < 0) {
    MAK_CUDA_TRY(cudaMemcpyAsync(&p, pdev, sizeof(int), cudaMemcpyDeviceToHost, st));
    MAK_CUDA_TRY(cudaStreamSynchronize(st));
  }

  // gauge tolerance: eps(max|dQ|)^(3/4) (0 for a zero tangent)
  if (gauge_atol >= 0) {
    Rr g = (Rr)gauge_atol;
    MAK_CUDA_TRY(cudaMemcpyAsync(gatol, &g, sizeof(Rr), cudaMemcpyHostToDevice, st));
    MAK_CUDA_TRY(cudaStreamSynchronize(st));
  } else if (dQ) {
    MAK_TRY(reduce_mat<T>(st, m, qc, dQ, lddq, 1, red, tmp));
    note_launch();
    eps34_kernel<Rr><<<1, 1, 0, st>>>(tmp, gatol);
    MAK_CUDA_TRY(cudaGetLastError());
  }

  // dQ1 (and the qr_full correction of the gauge-invariant part of dQ3)
  if (dQ) {
    MAK_TRY(copy_mat<T>(st, m, p, dQ, lddq, dQ1, m));
    if (p == k && qc > k) {
      const T* Q3 = Q + k * ldq;
      const T* dQ3src = dQ + k * lddq;
      MAK_TRY(copy_mat<T>(st, m, qc - k, dQ3src, lddq, dQ3, m));
      MAK_TRY(G(k, qc - k, m, one_<T>(), opnd<T>(Q, ldq, OP_C), opnd<T>(dQ3src, lddq), zero_<T>(),
                Q1dQ3, k));
      MAK_TRY(G(m, qc - k, k, -one_<T>(), opnd<T>(Q, ldq), opnd<T>(Q1dQ3, k), one_<T>(), dQ3, m));
      MAK_TRY(reduce_mat<T>(st, m, qc - k, dQ3, m, 1, red, gauge));
      MAK_TRY(G(m, k, qc - k, -one_<T>(), opnd<T>(Q3, ldq), opnd<T>(Q1dQ3, k, OP_C), one_<T>(),
                dQ1, m));
    } else if (qc > p) {
      MAK_TRY(reduce_mat<T>(st, m, qc - p, dQ + p * lddq, lddq, 1, red, gauge));
    }
  } else if (p > 0) {
    MAK_CUDA_TRY(cudaMemsetAsync(dQ1, 0, (size_t)m * p * sizeof(T), st));
  }
  if (dR && p < k) {
    note_launch();
    max_upper_kernel<T><<<64, 256, 0, st>>>((int)(k - p), (int)(n - p), dR + p + p * lddr, lddr,
                                            gauge);
    MAK_CUDA_TRY(cudaGetLastError());
  }

  if (p > 0) {
    const T* R12 = R + p * ldr;
    if (dR && n > p) {
      const T* dR12 = dR + p * lddr;
      // X = dR12 R12^H ; dQ1 -= Q1 X ; dA2 += Q1 dR12
      MAK_TRY(G(p, p, n - p, one_<T>(), opnd<T>(dR12, lddr), opnd<T>(R12, ldr, OP_C), zero_<T>(),
                X, p));
      MAK_TRY(G(m, p, p, -one_<T>(), opnd<T>(Q, ldq), opnd<T>(X, p), one_<T>(), dQ1, m));
      MAK_TRY(G(m, n - p, p, one_<T>(), opnd<T>(Q, ldq), opnd<T>(dR12, lddr), one_<T>(),
                dA + p * ldda, ldda));
    }
    // M = triu(dR11) R11^H - Q1^H dQ1
    if (dR)
      MAK_TRY(G(p, p, p, one_<T>(), opnd<T>(dR, lddr, OP_N, MASK_UPPER),
                opnd<T>(R, ldr, OP_C, MASK_UPPER), zero_<T>(), Mm, p));
    MAK_TRY(G(p, p, m, -one_<T>(), opnd<T>(Q, ldq, OP_C), opnd<T>(dQ1, m),
              dR ? one_<T>() : zero_<T>(), Mm, p));
    note_launch();
    copyltu_kernel<T><<<dim3((unsigned)ceil_div(p, 128), (unsigned)p), 128, 0, st>>>((int)p, Mm,
                                                                                      p);
    MAK_CUDA_TRY(cudaGetLastError());
    MAK_TRY(G(m, p, p, one_<T>(), opnd<T>(Q, ldq), opnd<T>(Mm, p), one_<T>(), dQ1, m));
    // dA1 += dQ1 R11^{-H}
    MAK_TRY(copy_mat<T>(st, p, p, R, ldr, X, p));
    {
      Arena gj(tail, tail_bytes);
      MAK_TRY(gje_inverse<T>(st, p, X, p, iperm, precision, gj, info));
    }
    note_launch();
    gather_cols_kernel<T><<<dim3((unsigned)ceil_div(p, 128), (unsigned)p), 128, 0, st>>>(
        (int)p, X, p, iperm, Rinv, p);
    MAK_CUDA_TRY(cudaGetLastError());
    MAK_TRY(G(m, p, p, one_<T>(), opnd<T>(dQ1, m), opnd<T>(Rinv, p, OP_C, MASK_UPPER), one_<T>(),
              dA, ldda));
  }
  note_launch();
  info_pullback_kernel<T><<<1, 1, 0, st>>>(info, p, 0, gauge, gatol);
  MAK_CUDA_TRY(cudaGetLastError());
  return 0;
}

// The numerical rank alone (reference qr_rank, src/pullbacks/qr.jl:1-2,
// tolerance eps(norm(R, Inf))^(3/4) when rank_atol < 0) into the device int
// *p_out: what qr_pullback_run computes first, for callers that read the
// ranks of many factorizations with one host synchronization.
template <class T>
int qr_rank_run(cudaStream_t st, int64_t k, int64_t n, const T* R, int64_t ldr, double rank_atol,
                Arena& ar, int* p_out) {
  using Rr = real_t<T>;
  Rr* scal = ar.take<Rr>(RED_CTAS + 4);
  if (ar.base == nullptr) return 0;
  if (!ar.ok()) return MAK_ERR_WORKSPACE;
  MAK_CUDA_TRY(cudaMemsetAsync(scal + RED_CTAS, 0, 4 * sizeof(Rr), st));
  MAK_TRY(reduce_mat<T>(st, k, n, R, ldr, 1, scal, scal + RED_CTAS));
  note_launch();
  qr_rank_kernel<T><<<1, 256, 0, st>>>((int)k, R, ldr, scal + RED_CTAS, rank_atol, p_out,
                                       scal + RED_CTAS + 1);
  return cudaGetLastError() == cudaSuccess ? 0 : MAK_ERR_CUDA;
}

#define MAK_INST_PB(T)                                                                         \
  template int qr_pullback_run<T>(cudaStream_t, int64_t, int64_t, int, T*, int64_t, const T*,  \
                                  int64_t, const T*, int64_t, const T*, int64_t, const T*,     \
                                  int64_t, double, double, int, Arena&, mak_info*, int);       \
  template int qr_rank_run<T>(cudaStream_t, int64_t, int64_t, const T*, int64_t, double,       \
                              Arena&, int*);
MAK_INST_PB(double)
MAK_INST_PB(zcomplex)
MAK_INST_PB(float)
MAK_INST_PB(ccomplex)

// ----------------------------------------------------------- polar pullback --
// Scratch of the device Sylvester solve (and of the products around it).
template <class T>
struct SylScratch {
  real_t<T>* scal;
  T *Mm, *Ak, *Ck, *Ai, *Tm, *Y, *Pinv;
  int* iperm;
  int* stopw;  // device stop of the sign iteration: [0] stop flag, [1] iterations
  char* tail;
  size_t tail_bytes;
};
template <class T>
static SylScratch<T> syl_take(Arena& ar, cudaStream_t st, int64_t m, int64_t n, int precision) {
  using Rr = real_t<T>;
  const size_t nn = (size_t)n * n;
  SylScratch<T> s;
  s.scal = ar.take<Rr>(RED_CTAS + 16);
  s.Mm = ar.take<T>(nn + 1);
  s.Ak = ar.take<T>(nn + 1);
  s.Ck = ar.take<T>(nn + 1);
  s.Ai = ar.take<T>(nn + 1);
  s.Pinv = ar.take<T>(nn + 1);
  s.Tm = ar.take<T>(nn + 1);
  s.Y = ar.take<T>((size_t)m * n + 1);
  s.iperm = ar.take<int>(n + 1);
  s.stopw = ar.take<int>(2);
  size_t gj_ws = 0, oz_ws = 0;
  {
    Arena meas(nullptr, 0);
    gje_inverse<T>(st, n, nullptr, n, nullptr, precision, meas, nullptr);
    gj_ws = meas.off + 256;
    const int64_t shapes[3][3] = {{n, n, m}, {n, n, n}, {m, n, n}};
    for (auto& sh : shapes) {
      Arena m2(nullptr, 0);
      gemm_prec<T>(st, precision, sh[0], sh[1], sh[2], one_<T>(), opnd<T>(nullptr, 1),
                   opnd<T>(nullptr, 1), zero_<T>(), nullptr, 1, m2, nullptr);
      if (m2.off + 256 > oz_ws) oz_ws = m2.off + 256;
    }
  }
  s.tail_bytes = gj_ws > oz_ws ? gj_ws : oz_ws;
  s.tail = ar.take<char>(s.tail_bytes);
  return s;
}

// Solves P X + X P = M - M^H for X (n x n, ld n) with P Hermitian positive
// definite, by the sign-function Newton iteration on [[P, -C], [0, -P]]
// carried on its two blocks (A_k, C_k): A_{k+1} = (A_k + A_k^-1)/2,
// C_{k+1} = (C_k + A_k^-1 C_k A_k^-1)/2 from A_0 = P, C_0 = -(M - M^H);
// the solution is X = -C_inf / 2.  M is read from s.Mm (ld n); P^-1 (the
// first iterate's inverse) is left in s.Pinv; X goes to s.Tm.  maxiter > 0:
// the host synchronizes once per iteration for the stopping test.
// maxiter < 0: no host synchronization (CUDA-graph capturable): -maxiter
// iterations are launched and the loop stops on the device once the test
// is met (the stopped iterations' kernels return at once); *iters is then
// -1 and the count and the outcome stay in s.stopw.
template <class T>
static int syl_solve(cudaStream_t st, int64_t n, const T* P, int64_t ldp, int maxiter,
                     int precision, SylScratch<T>& s, mak_info* info, int* iters) {
  using Rr = real_t<T>;
  const size_t nn = (size_t)n * n;
  const bool fixed = maxiter < 0;
  if (fixed) maxiter = -maxiter;
  int* status = &info->status;
  Rr* red = s.scal;
  Rr* nrm2 = s.scal + RED_CTAS;  // [0] ||A||^2, [1] ||Ai||^2, [2] ||dA||^2
  auto G = [&](int64_t M_, int64_t N_, int64_t K_, T alpha, Operand<T> a, Operand<T> b, T beta,
               T* C_, int64_t ldc) -> int {
    Arena oz(s.tail, s.tail_bytes);
    return gemm_prec<T>(st, precision, M_, N_, K_, alpha, a, b, beta, C_, ldc, oz, status);
  };
  auto inverse = [&](const T* X, T* out) -> int {
    MAK_TRY(copy_mat<T>(st, n, n, X, n, s.Tm, n));
    {
      Arena gj(s.tail, s.tail_bytes);
      MAK_TRY(gje_inverse<T>(st, n, s.Tm, n, s.iperm, precision, gj, info));
    }
    note_launch();
    gather_cols_kernel<T><<<dim3((unsigned)ceil_div(n, 128), (unsigned)n), 128, 0, st>>>(
        (int)n, s.Tm, n, s.iperm, out, n);
    return cudaGetLastError() == cudaSuccess ? 0 : MAK_ERR_CUDA;
  };
  const unsigned g1 = (unsigned)ceil_div((int64_t)nn, 256);
  // C_0 = -(M - M^H), A_0 = P
  {
    dim3 g((unsigned)ceil_div(n, 32), (unsigned)ceil_div(n, 32));
    note_launch();
    antiherm_kernel<T><<<g, 256, 0, st>>>((int)n, s.Mm, n, Rr(-1), s.Ck, n);
    MAK_CUDA_TRY(cudaGetLastError());
  }
  MAK_TRY(copy_mat<T>(st, n, n, P, ldp, s.Ak, n));
  const Rr tol = (sizeof(Rr) == 8 ? Rr(1e-13) : Rr(1e-6)) * sqrt((Rr)n);
  int it = 0;
  if (fixed) MAK_CUDA_TRY(cudaMemsetAsync(s.stopw, 0, 2 * sizeof(int), st));
  for (it = 1; it <= maxiter; it++) {
    SkipScope skip(fixed ? s.stopw : skip_flag());
    MAK_TRY(inverse(s.Ak, s.Ai));
    if (it == 1) MAK_TRY(copy_mat<T>(st, n, n, s.Ai, n, s.Pinv, n));
    MAK_TRY(reduce_mat<T>(st, n, n, s.Ak, n, 0, red, nrm2));
    MAK_TRY(reduce_mat<T>(st, n, n, s.Ai, n, 0, red, nrm2 + 1));
    // Tm = Ai C Ai
    MAK_TRY(G(n, n, n, one_<T>(), opnd<T>(s.Ai, n), opnd<T>(s.Ck, n), zero_<T>(), s.Y, n));
    MAK_TRY(G(n, n, n, one_<T>(), opnd<T>(s.Y, n), opnd<T>(s.Ai, n), zero_<T>(), s.Tm, n));
    const unsigned gr = g1 < RED_CTAS ? g1 : RED_CTAS;
    note_launch();
    sign_update_kernel<T><<<gr, 256, 0, st>>>((int64_t)nn, s.Ak, s.Ai, s.Ck, s.Tm, nrm2, red,
                                               skip_flag());
    MAK_CUDA_TRY(cudaGetLastError());
    note_launch();
    reduce_final_kernel<Rr><<<1, 256, 0, st>>>((int)gr, red, 0, nrm2 + 2);
    MAK_CUDA_TRY(cudaGetLastError());
    MAK_TRY(herm_project<T>(st, n, s.Ak, n));  // idempotent once A is Hermitian
    if (fixed) {
      note_launch();
      sign_stop_kernel<Rr><<<1, 1, 0, st>>>(nrm2 + 2, tol, s.stopw);
      MAK_CUDA_TRY(cudaGetLastError());
      continue;
    }
    Rr dnorm2 = 0;
    MAK_CUDA_TRY(cudaMemcpyAsync(&dnorm2, nrm2 + 2, sizeof(Rr), cudaMemcpyDeviceToHost, st));
    MAK_CUDA_TRY(cudaStreamSynchronize(st));
    if (!(sqrt(dnorm2) > tol)) break;
  }
  if (it > maxiter) it = maxiter;
  *iters = fixed ? -1 : it;
  // X = -C_inf / 2
  note_launch();
  scale_copy_kernel<T><<<g1, 256, 0, st>>>((int64_t)nn, s.Ck, Rr(-0.5), s.Tm);
  return cudaGetLastError() == cudaSuccess ? 0 : MAK_ERR_CUDA;
}

template <class T>
int polar_pullback_run(cudaStream_t st, int64_t m, int64_t n, T* dA, int64_t ldda, const T* W,
                       int64_t ldw, const T* P, int64_t ldp, const T* dW, int64_t lddw,
                       const T* dP, int64_t lddp, int maxiter, int precision, Arena& ar,
                       mak_info* info) {
  const size_t nn = (size_t)n * n;
  T* dPh = ar.take<T>(nn + 1);
  SylScratch<T> s = syl_take<T>(ar, st, m, n, precision);
  if (ar.base == nullptr) return 0;
  if (!ar.ok()) return MAK_ERR_WORKSPACE;
  if (n == 0) return 0;
  int* status = &info->status;
  auto G = [&](int64_t M_, int64_t N_, int64_t K_, T alpha, Operand<T> a, Operand<T> b, T beta,
               T* C_, int64_t ldc) -> int {
    Arena oz(s.tail, s.tail_bytes);
    return gemm_prec<T>(st, precision, M_, N_, K_, alpha, a, b, beta, C_, ldc, oz, status);
  };
  const unsigned g1 = (unsigned)ceil_div((int64_t)nn, 256);

  // dP <- herm(dP);  M = W^H dW - dP P
  if (dP) {
    MAK_TRY(copy_mat<T>(st, n, n, dP, lddp, dPh, n));
    MAK_TRY(herm_project<T>(st, n, dPh, n));
  }
  if (dW)
    MAK_TRY(G(n, n, m, one_<T>(), opnd<T>(W, ldw, OP_C), opnd<T>(dW, lddw), zero_<T>(), s.Mm, n));
  else
    MAK_CUDA_TRY(cudaMemsetAsync(s.Mm, 0, nn * sizeof(T), st));
  if (dP)
    MAK_TRY(G(n, n, n, -one_<T>(), opnd<T>(dPh, n), opnd<T>(P, ldp), one_<T>(), s.Mm, n));
  // C = sylvester(P, P, M^H - M):  P C + C P = M - M^H
  int it = 0;
  MAK_TRY(syl_solve<T>(st, n, P, ldp, maxiter, precision, s, info, &it));
  if (dP) {
    note_launch();
    add_kernel<T><<<g1, 256, 0, st>>>((int64_t)nn, dPh, s.Tm);
    MAK_CUDA_TRY(cudaGetLastError());
  }
  // dA += W C
  MAK_TRY(G(m, n, n, one_<T>(), opnd<T>(W, ldw), opnd<T>(s.Tm, n), one_<T>(), dA, ldda));
  // dA += (I - W W^H) dW P^{-1}
  if (dW) {
    MAK_TRY(G(m, n, n, one_<T>(), opnd<T>(dW, lddw), opnd<T>(s.Pinv, n), zero_<T>(), s.Y, m));
    MAK_TRY(G(n, n, m, one_<T>(), opnd<T>(W, ldw, OP_C), opnd<T>(s.Y, m), zero_<T>(), s.Mm, n));
    MAK_TRY(G(m, n, n, -one_<T>(), opnd<T>(W, ldw), opnd<T>(s.Mm, n), one_<T>(), s.Y, m));
    {
      dim3 g((unsigned)ceil_div(m, 256), (unsigned)(n < 65535 ? n : 65535));
      note_launch();
      add_strided_kernel<T><<<g, 256, 0, st>>>(m, n, s.Y, m, dA, ldda);
      MAK_CUDA_TRY(cudaGetLastError());
    }
  }
  note_launch();
  info_pullback_kernel<T><<<1, 1, 0, st>>>(info, (int)n, it, nullptr, nullptr);
  MAK_CUDA_TRY(cudaGetLastError());
  if (it < 0) {
    note_launch();
    info_sign_fixed_kernel<<<1, 1, 0, st>>>(info, s.stopw);
    MAK_CUDA_TRY(cudaGetLastError());
  }
  return 0;
}

// left_polar_pushforward!: the tangent (dW, dP) of the left polar
// decomposition A = W P along dA (reference src/pushforwards/polar.jl:1-12):
//   dP0 = W^H dA,  K = sylvester(P, P, dP0^H - dP0)  (P K + K P = dP0 - dP0^H),
//   dW = (I - W W^H) dA P^-1 + W K,  dP = dP0 - K P.
// dW (m x n) and dP (n x n) are outputs (overwritten).
template <class T>
int polar_pushforward_run(cudaStream_t st, int64_t m, int64_t n, const T* dA, int64_t ldda,
                          const T* W, int64_t ldw, const T* P, int64_t ldp, T* dW, int64_t lddw,
                          T* dP, int64_t lddp, int maxiter, int precision, Arena& ar,
                          mak_info* info) {
  SylScratch<T> s = syl_take<T>(ar, st, m, n, precision);
  if (ar.base == nullptr) return 0;
  if (!ar.ok()) return MAK_ERR_WORKSPACE;
  if (n == 0) return 0;
  int* status = &info->status;
  auto G = [&](int64_t M_, int64_t N_, int64_t K_, T alpha, Operand<T> a, Operand<T> b, T beta,
               T* C_, int64_t ldc) -> int {
    Arena oz(s.tail, s.tail_bytes);
    return gemm_prec<T>(st, precision, M_, N_, K_, alpha, a, b, beta, C_, ldc, oz, status);
  };
  // dP = W^H dA (kept for the end), M = the same
  MAK_TRY(G(n, n, m, one_<T>(), opnd<T>(W, ldw, OP_C), opnd<T>(dA, ldda), zero_<T>(), dP, lddp));
  MAK_TRY(copy_mat<T>(st, n, n, dP, lddp, s.Mm, n));
  int it = 0;
  MAK_TRY(syl_solve<T>(st, n, P, ldp, maxiter, precision, s, info, &it));  // K in s.Tm
  // dW = dA P^-1;  dW -= W (W^H dW);  dW += W K
  MAK_TRY(G(m, n, n, one_<T>(), opnd<T>(dA, ldda), opnd<T>(s.Pinv, n), zero_<T>(), dW, lddw));
  MAK_TRY(G(n, n, m, one_<T>(), opnd<T>(W, ldw, OP_C), opnd<T>(dW, lddw), zero_<T>(), s.Mm, n));
  MAK_TRY(G(m, n, n, -one_<T>(), opnd<T>(W, ldw), opnd<T>(s.Mm, n), one_<T>(), dW, lddw));
  MAK_TRY(G(m, n, n, one_<T>(), opnd<T>(W, ldw), opnd<T>(s.Tm, n), one_<T>(), dW, lddw));
  // dP -= K P
  MAK_TRY(G(n, n, n, -one_<T>(), opnd<T>(s.Tm, n), opnd<T>(P, ldp), one_<T>(), dP, lddp));
  note_launch();
  info_pullback_kernel<T><<<1, 1, 0, st>>>(info, (int)n, it, nullptr, nullptr);
  MAK_CUDA_TRY(cudaGetLastError());
  return 0;
}

#define MAK_INST_PPB(T)                                                                        \
  template int polar_pullback_run<T>(cudaStream_t, int64_t, int64_t, T*, int64_t, const T*,    \
                                     int64_t, const T*, int64_t, const T*, int64_t, const T*,  \
                                     int64_t, int, int, Arena&, mak_info*);
MAK_INST_PPB(double)
MAK_INST_PPB(zcomplex)
MAK_INST_PPB(float)
MAK_INST_PPB(ccomplex)

constexpr int SIGN_MAXITER = 60;

template <class T>
static int qr_pullback_entry(int64_t m, int64_t n, int full, void* dAv, int64_t ldda,
                             const void* Qv, int64_t ldq, const void* Rv, int64_t ldr,
                             const void* dQv, int64_t lddq, const void* dRv, int64_t lddr,
                             const mak_pullback_opts* opts, void* work, size_t work_bytes,
                             mak_info* info, mak_stream_t stream) {
  const int64_t k = m < n ? m : n;
  const int64_t qc = full ? m : k, rr = full ? m : k;
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (dAv == nullptr && m * n > 0) return -4;
  if (ldda < (m > 1 ? m : 1)) return -5;
  if (Qv == nullptr && m * qc > 0) return -6;
  if (ldq < (m > 1 ? m : 1)) return -7;
  if (Rv == nullptr && rr * n > 0) return -8;
  if (ldr < (rr > 1 ? rr : 1)) return -9;
  if (dQv && lddq < (m > 1 ? m : 1)) return -11;
  if (dRv && lddr < (rr > 1 ? rr : 1)) return -13;
  mak_pullback_opts o{-1.0, -1.0, MAK_PREC_NATIVE, 0};
  if (opts) o = *opts;
  if (o.precision != MAK_PREC_NATIVE && o.precision != MAK_PREC_MIXED) return -14;
  if (info == nullptr) return -17;
  cudaStream_t st = (cudaStream_t)stream;
  {
    Arena meas(nullptr, 0);
    qr_pullback_run<T>(st, m, n, full, nullptr, ldda, nullptr, ldq, nullptr, ldr, nullptr, lddq,
                       nullptr, lddr, o.rank_atol, o.gauge_atol, o.precision, meas, nullptr);
    if (meas.off > work_bytes) return -16;
  }
  MAK_TRY(info_reset(st, info));
  Arena ar(work, work_bytes);
  return qr_pullback_run<T>(st, m, n, full, (T*)dAv, ldda, (const T*)Qv, ldq, (const T*)Rv, ldr,
                            (const T*)dQv, lddq, (const T*)dRv, lddr, o.rank_atol, o.gauge_atol,
                            o.precision, ar, info);
}

template <class T>
static int polar_pullback_entry(int64_t m, int64_t n, void* dAv, int64_t ldda, const void* Wv,
                                int64_t ldw, const void* Pv, int64_t ldp, const void* dWv,
                                int64_t lddw, const void* dPv, int64_t lddp,
                                const mak_pullback_opts* opts, void* work, size_t work_bytes,
                                mak_info* info, mak_stream_t stream) {
  if (m < 0) return -1;
  if (n < 0 || n > m) return -2;
  if (dAv == nullptr && m * n > 0) return -3;
  if (ldda < (m > 1 ? m : 1)) return -4;
  if (Wv == nullptr && m * n > 0) return -5;
  if (ldw < (m > 1 ? m : 1)) return -6;
  if (Pv == nullptr && n > 0) return -7;
  if (ldp < (n > 1 ? n : 1)) return -8;
  if (dWv && lddw < (m > 1 ? m : 1)) return -10;
  if (dPv && lddp < (n > 1 ? n : 1)) return -12;
  mak_pullback_opts o{-1.0, -1.0, MAK_PREC_NATIVE, 0};
  if (opts) o = *opts;
  if (o.precision != MAK_PREC_NATIVE && o.precision != MAK_PREC_MIXED) return -13;
  if (info == nullptr) return -16;
  cudaStream_t st = (cudaStream_t)stream;
  {
    Arena meas(nullptr, 0);
    polar_pullback_run<T>(st, m, n, nullptr, ldda, nullptr, ldw, nullptr, ldp, nullptr, lddw,
                          nullptr, lddp, SIGN_MAXITER, o.precision, meas, nullptr);
    if (meas.off > work_bytes) return -15;
  }
  MAK_TRY(info_reset(st, info));
  Arena ar(work, work_bytes);
  return polar_pullback_run<T>(st, m, n, (T*)dAv, ldda, (const T*)Wv, ldw, (const T*)Pv, ldp,
                               (const T*)dWv, lddw, (const T*)dPv, lddp, SIGN_MAXITER,
                               o.precision, ar, info);
}

template <class T>
static int polar_pushforward_entry(int64_t m, int64_t n, const void* dAv, int64_t ldda,
                                   const void* Wv, int64_t ldw, const void* Pv, int64_t ldp,
                                   void* dWv, int64_t lddw, void* dPv, int64_t lddp,
                                   const mak_pullback_opts* opts, void* work, size_t work_bytes,
                                   mak_info* info, mak_stream_t stream) {
  if (m < 0) return -1;
  if (n < 0 || n > m) return -2;
  if (dAv == nullptr && m * n > 0) return -3;
  if (ldda < (m > 1 ? m : 1)) return -4;
  if (Wv == nullptr && m * n > 0) return -5;
  if (ldw < (m > 1 ? m : 1)) return -6;
  if (Pv == nullptr && n > 0) return -7;
  if (ldp < (n > 1 ? n : 1)) return -8;
  if (dWv == nullptr && m * n > 0) return -9;
  if (lddw < (m > 1 ? m : 1)) return -10;
  if (dPv == nullptr && n > 0) return -11;
  if (lddp < (n > 1 ? n : 1)) return -12;
  mak_pullback_opts o{-1.0, -1.0, MAK_PREC_NATIVE, 0};
  if (opts) o = *opts;
  if (o.precision != MAK_PREC_NATIVE && o.precision != MAK_PREC_MIXED) return -13;
  if (info == nullptr) return -16;
  cudaStream_t st = (cudaStream_t)stream;
  {
    Arena meas(nullptr, 0);
    polar_pushforward_run<T>(st, m, n, nullptr, ldda, nullptr, ldw, nullptr, ldp, nullptr, lddw,
                             nullptr, lddp, SIGN_MAXITER, o.precision, meas, nullptr);
    if (meas.off > work_bytes) return -15;
  }
  MAK_TRY(info_reset(st, info));
  Arena ar(work, work_bytes);
  return polar_pushforward_run<T>(st, m, n, (const T*)dAv, ldda, (const T*)Wv, ldw,
                                  (const T*)Pv, ldp, (T*)dWv, lddw, (T*)dPv, lddp, SIGN_MAXITER,
                                  o.precision, ar, info);
}

// right_polar_pullback! (reference src/pullbacks/polar.jl:37-59) as the left
// pullback of A^H: right_polar(A) = (P, Wh) is left_polar(A^H) = (Wh^H, P),
// and the cotangent pairing is preserved by the conjugate transpose, so
// dA += (left_polar_pullback of A^H at (Wh^H, P) with (dWh^H, dP))^H.
template <class T>
static int right_polar_pullback_run(cudaStream_t st, int64_t m, int64_t n, T* dA, int64_t ldda,
                                    const T* P, int64_t ldp, const T* Wh, int64_t ldwh,
                                    const T* dP, int64_t lddp, const T* dWh, int64_t lddwh,
                                    int precision, Arena& ar, mak_info* info) {
  T* Wt = ar.take<T>((size_t)n * m + 1);
  T* dWt = ar.take<T>((size_t)n * m + 1);
  T* dB = ar.take<T>((size_t)n * m + 1);
  size_t inner = 0;
  {
    Arena meas(nullptr, 0);
    polar_pullback_run<T>(st, n, m, nullptr, n, nullptr, n, nullptr, m, nullptr, n, nullptr, m,
                          SIGN_MAXITER, precision, meas, nullptr);
    inner = meas.off + 256;
  }
  char* sub = ar.take<char>(inner);
  if (ar.base == nullptr) return 0;
  if (!ar.ok()) return MAK_ERR_WORKSPACE;
  if (m == 0 || n == 0) return 0;
  MAK_TRY(ctranspose<T>(st, m, n, Wh, ldwh, Wt, n));
  if (dWh) MAK_TRY(ctranspose<T>(st, m, n, dWh, lddwh, dWt, n));
  MAK_CUDA_TRY(cudaMemsetAsync(dB, 0, (size_t)n * m * sizeof(T), st));
  Arena a2(sub, inner);
  MAK_TRY(polar_pullback_run<T>(st, n, m, dB, n, Wt, n, P, ldp, dWh ? dWt : nullptr, n, dP, lddp,
                                SIGN_MAXITER, precision, a2, info));
  return ctranspose<T>(st, n, m, dB, n, dA, ldda, true);
}

template <class T>
static int right_polar_pullback_entry(int64_t m, int64_t n, void* dAv, int64_t ldda,
                                      const void* Pv, int64_t ldp, const void* Whv, int64_t ldwh,
                                      const void* dPv, int64_t lddp, const void* dWhv,
                                      int64_t lddwh, const mak_pullback_opts* opts, void* work,
                                      size_t work_bytes, mak_info* info, mak_stream_t stream) {
  if (m < 0) return -1;
  if (n < m) return -2;
  if (dAv == nullptr && m * n > 0) return -3;
  if (ldda < (m > 1 ? m : 1)) return -4;
  if (Pv == nullptr && m > 0) return -5;
  if (ldp < (m > 1 ? m : 1)) return -6;
  if (Whv == nullptr && m * n > 0) return -7;
  if (ldwh < (m > 1 ? m : 1)) return -8;
  if (dPv && lddp < (m > 1 ? m : 1)) return -10;
  if (dWhv && lddwh < (m > 1 ? m : 1)) return -12;
  mak_pullback_opts o{-1.0, -1.0, MAK_PREC_NATIVE, 0};
  if (opts) o = *opts;
  if (o.precision != MAK_PREC_NATIVE && o.precision != MAK_PREC_MIXED) return -13;
  if (info == nullptr) return -16;
  cudaStream_t st = (cudaStream_t)stream;
  {
    Arena meas(nullptr, 0);
    right_polar_pullback_run<T>(st, m, n, nullptr, ldda, nullptr, ldp, nullptr, ldwh, nullptr,
                                lddp, nullptr, lddwh, o.precision, meas, nullptr);
    if (meas.off > work_bytes) return -15;
  }
  MAK_TRY(info_reset(st, info));
  Arena ar(work, work_bytes);
  return right_polar_pullback_run<T>(st, m, n, (T*)dAv, ldda, (const T*)Pv, ldp, (const T*)Whv,
                                     ldwh, (const T*)dPv, lddp, (const T*)dWhv, lddwh,
                                     o.precision, ar, info);
}

// right_polar_pushforward! (reference src/pushforwards/polar.jl:14-26) as the
// left pushforward of A^H at (Wh^H, P) along dA^H: the returned tangents are
// the conjugate transposes (dWh = dW'^H, dP = dP'^H).  m <= n.
template <class T>
static int right_polar_pushforward_run(cudaStream_t st, int64_t m, int64_t n, const T* dA,
                                       int64_t ldda, const T* P, int64_t ldp, const T* Wh,
                                       int64_t ldwh, T* dP, int64_t lddp, T* dWh, int64_t lddwh,
                                       int precision, Arena& ar, mak_info* info) {
  T* dAt = ar.take<T>((size_t)n * m + 1);
  T* Wt = ar.take<T>((size_t)n * m + 1);
  T* dWt = ar.take<T>((size_t)n * m + 1);
  T* dPt = ar.take<T>((size_t)m * m + 1);
  size_t inner = 0;
  {
    Arena meas(nullptr, 0);
    polar_pushforward_run<T>(st, n, m, nullptr, n, nullptr, n, nullptr, m, nullptr, n, nullptr, m,
                             SIGN_MAXITER, precision, meas, nullptr);
    inner = meas.off + 256;
  }
  char* sub = ar.take<char>(inner);
  if (ar.base == nullptr) return 0;
  if (!ar.ok()) return MAK_ERR_WORKSPACE;
  if (m == 0 || n == 0) return 0;
  MAK_TRY(ctranspose<T>(st, m, n, dA, ldda, dAt, n));
  MAK_TRY(ctranspose<T>(st, m, n, Wh, ldwh, Wt, n));
  Arena a2(sub, inner);
  MAK_TRY(polar_pushforward_run<T>(st, n, m, dAt, n, Wt, n, P, ldp, dWt, n, dPt, m, SIGN_MAXITER,
                                   precision, a2, info));
  MAK_TRY(ctranspose<T>(st, n, m, dWt, n, dWh, lddwh));
  return ctranspose<T>(st, m, m, dPt, m, dP, lddp);
}

template <class T>
static int right_polar_pushforward_entry(int64_t m, int64_t n, const void* dAv, int64_t ldda,
                                         const void* Pv, int64_t ldp, const void* Whv,
                                         int64_t ldwh, void* dPv, int64_t lddp, void* dWhv,
                                         int64_t lddwh, const mak_pullback_opts* opts, void* work,
                                         size_t work_bytes, mak_info* info, mak_stream_t stream) {
  if (m < 0) return -1;
  if (n < m) return -2;
  if (dAv == nullptr && m * n > 0) return -3;
  if (ldda < (m > 1 ? m : 1)) return -4;
  if (Pv == nullptr && m > 0) return -5;
  if (ldp < (m > 1 ? m : 1)) return -6;
  if (Whv == nullptr && m * n > 0) return -7;
  if (ldwh < (m > 1 ? m : 1)) return -8;
  if (dPv == nullptr && m > 0) return -9;
  if (lddp < (m > 1 ? m : 1)) return -10;
  if (dWhv == nullptr && m * n > 0) return -11;
  if (lddwh < (m > 1 ? m : 1)) return -12;
  mak_pullback_opts o{-1.0, -1.0, MAK_PREC_NATIVE, 0};
  if (opts) o = *opts;
  if (o.precision != MAK_PREC_NATIVE && o.precision != MAK_PREC_MIXED) return -13;
  if (info == nullptr) return -16;
  cudaStream_t st = (cudaStream_t)stream;
  {
    Arena meas(nullptr, 0);
    right_polar_pushforward_run<T>(st, m, n, nullptr, ldda, nullptr, ldp, nullptr, ldwh, nullptr,
                                   lddp, nullptr, lddwh, o.precision, meas, nullptr);
    if (meas.off > work_bytes) return -15;
  }
  MAK_TRY(info_reset(st, info));
  Arena ar(work, work_bytes);
  return right_polar_pushforward_run<T>(st, m, n, (const T*)dAv, ldda, (const T*)Pv, ldp,
                                        (const T*)Whv, ldwh, (T*)dPv, lddp, (T*)dWhv, lddwh,
                                        o.precision, ar, info);
}

template <class T>
static size_t rpolar_pf_ws(int64_t m, int64_t n, int prec) {
  Arena meas(nullptr, 0);
  right_polar_pushforward_run<T>(0, m, n, nullptr, m, nullptr, m, nullptr, m, nullptr, m, nullptr,
                                 m, prec, meas, nullptr);
  return meas.off + 256;
}

template <class T>
static size_t polar_pf_ws(int64_t m, int64_t n, int prec) {
  Arena meas(nullptr, 0);
  polar_pushforward_run<T>(0, m, n, nullptr, m, nullptr, m, nullptr, n, nullptr, m, nullptr, n,
                           SIGN_MAXITER, prec, meas, nullptr);
  return meas.off + 256;
}
template <class T>
static size_t rpolar_pb_ws(int64_t m, int64_t n, int prec) {
  Arena meas(nullptr, 0);
  right_polar_pullback_run<T>(0, m, n, nullptr, m, nullptr, m, nullptr, m, nullptr, m, nullptr,
                              m, prec, meas, nullptr);
  return meas.off + 256;
}

// ------------------------------------------------ null-space and LQ pullbacks --
template <class R>
__global__ void sqrt_scalar_kernel(const R* x, R* out) {
  *out = sqrt(*x);
}

// qr_null_pullback! (reference src/pullbacks/qr.jl:141-152) for N = qr_null(A)
// (m x (m-n), nonempty only for m > n) and a nonzero cotangent dN:
//   gauge = ||(S - S^H)/2||_F with S = N^H dN (check_qr_null_cotangents,
//   qr.jl:122-128; reported in info->gauge against info->gauge_atol),
//   Q, R = qr_compact(A; positive = true),  X = (dN^H Q) R^{-H},  dA -= N X.
// R^{-1} is the explicit Gauss-Jordan inverse of the triangular factor (no
// pivot exchanges occur on a triangular matrix).  A is read, not written.
template <class T>
static int qr_null_pullback_run(cudaStream_t st, int64_t m, int64_t n, T* dA, int64_t ldda,
                                const T* A, int64_t lda, const T* N, int64_t ldn, const T* dN,
                                int64_t lddn, double gauge_atol, int precision, Arena& ar,
                                mak_info* info) {
  using Rr = real_t<T>;
  const int64_t k = m < n ? m : n;
  const int64_t nc = m - k;
  Rr* scal = ar.take<Rr>(RED_CTAS + 16);
  T* Ac = ar.take<T>((size_t)m * n + 1);
  T* Qc = ar.take<T>((size_t)m * k + 1);
  T* Rc = ar.take<T>((size_t)k * k + 1);  // R is k x n = k x k whenever nc > 0
  T* S = ar.take<T>((size_t)nc * nc + 1);
  T* Sa = ar.take<T>((size_t)nc * nc + 1);
  T* G1 = ar.take<T>((size_t)nc * k + 1);
  T* X = ar.take<T>((size_t)nc * k + 1);
  T* Rinv = ar.take<T>((size_t)k * k + 1);
  int* iperm = ar.take<int>(k + 1);
  size_t tail_bytes = 0;
  {
    Arena mq(nullptr, 0);
    qr_run<T>(st, m, n, nullptr, m > 0 ? m : 1, nullptr, m > 0 ? m : 1, k, nullptr,
              k > 0 ? k : 1, k, 1, 0, precision, mq, nullptr);
    tail_bytes = mq.off + 256;
    Arena mg(nullptr, 0);
    gje_inverse<T>(st, k, nullptr, k > 0 ? k : 1, nullptr, precision, mg, nullptr);
    if (mg.off + 256 > tail_bytes) tail_bytes = mg.off + 256;
    const int64_t shapes[4][3] = {{nc, nc, m}, {nc, k, m}, {nc, k, k}, {m, k, nc}};
    for (auto& sh : shapes) {
      Arena m2(nullptr, 0);
      gemm_prec<T>(st, precision, sh[0], sh[1], sh[2], one_<T>(), opnd<T>(nullptr, 1),
                   opnd<T>(nullptr, 1), zero_<T>(), nullptr, 1, m2, nullptr);
      if (m2.off + 256 > tail_bytes) tail_bytes = m2.off + 256;
    }
  }
  char* tail = ar.take<char>(tail_bytes);
  if (ar.base == nullptr) return 0;
  if (!ar.ok()) return MAK_ERR_WORKSPACE;
  int* status = &info->status;
  Rr* red = scal;
  Rr* gauge = scal + RED_CTAS;
  Rr* gatol = scal + RED_CTAS + 1;
  Rr* tmp = scal + RED_CTAS + 2;
  auto G = [&](int64_t M_, int64_t N_, int64_t K_, T alpha, Operand<T> a, Operand<T> b, T beta,
               T* C_, int64_t ldc) -> int {
    Arena oz(tail, tail_bytes);
    return gemm_prec<T>(st, precision, M_, N_, K_, alpha, a, b, beta, C_, ldc, oz, status);
  };
  MAK_CUDA_TRY(cudaMemsetAsync(scal + RED_CTAS, 0, 16 * sizeof(Rr), st));
  if (dN != nullptr && nc > 0) {
    // gauge check of the cotangent
    MAK_TRY(G(nc, nc, m, one_<T>(), opnd<T>(N, ldn, OP_C), opnd<T>(dN, lddn), zero_<T>(), S, nc));
    {
      dim3 g((unsigned)ceil_div(nc, 32), (unsigned)ceil_div(nc, 32));
      note_launch();
      antiherm_kernel<T><<<g, 256, 0, st>>>((int)nc, S, nc, Rr(0.5), Sa, nc);
      MAK_CUDA_TRY(cudaGetLastError());
    }
    MAK_TRY(reduce_mat<T>(st, nc, nc, Sa, nc, 0, red, tmp));
    note_launch();
    sqrt_scalar_kernel<Rr><<<1, 1, 0, st>>>(tmp, gauge);
    MAK_CUDA_TRY(cudaGetLastError());
    if (gauge_atol >= 0) {
      Rr g = (Rr)gauge_atol;
      MAK_CUDA_TRY(cudaMemcpyAsync(gatol, &g, sizeof(Rr), cudaMemcpyHostToDevice, st));
      MAK_CUDA_TRY(cudaStreamSynchronize(st));
    } else {
      MAK_TRY(reduce_mat<T>(st, m, nc, dN, lddn, 1, red, tmp));
      note_launch();
      eps34_kernel<Rr><<<1, 1, 0, st>>>(tmp, gatol);
      MAK_CUDA_TRY(cudaGetLastError());
    }
    if (k > 0) {
      // Q, R of A (positive gauge)
      MAK_TRY(copy_mat<T>(st, m, n, A, lda, Ac, m));
      {
        Arena qa(tail, tail_bytes);
        MAK_TRY(qr_run<T>(st, m, n, Ac, m, Qc, m, k, Rc, k, k, 1, 0, precision, qa, info));
      }
      // G1 = dN^H Q;  R^{-1};  X = G1 R^{-H};  dA -= N X
      MAK_TRY(G(nc, k, m, one_<T>(), opnd<T>(dN, lddn, OP_C), opnd<T>(Qc, m), zero_<T>(), G1, nc));
      {
        Arena gj(tail, tail_bytes);
        MAK_TRY(gje_inverse<T>(st, k, Rc, k, iperm, precision, gj, info));
      }
      note_launch();
      gather_cols_kernel<T><<<dim3((unsigned)ceil_div(k, 128), (unsigned)k), 128, 0, st>>>(
          (int)k, Rc, k, iperm, Rinv, k);
      MAK_CUDA_TRY(cudaGetLastError());
      MAK_TRY(G(nc, k, k, one_<T>(), opnd<T>(G1, nc), opnd<T>(Rinv, k, OP_C, MASK_UPPER),
                zero_<T>(), X, nc));
      MAK_TRY(G(m, k, nc, -one_<T>(), opnd<T>(N, ldn), opnd<T>(X, nc), one_<T>(), dA, ldda));
    }
  }
  note_launch();
  info_pullback_kernel<T><<<1, 1, 0, st>>>(info, (int)k, 0, gauge, gatol);
  MAK_CUDA_TRY(cudaGetLastError());
  return 0;
}

// lq_pullback! (reference src/pullbacks/lq.jl:71-112) is the conjugate
// transpose of qr_pullback! of A^H at (Q^H, L^H) with cotangents (dQ^H, dL^H):
// the rank test, the gauge measures (max-abs norms) and every product of the
// reference's LQ rule are the QR rule's, transposed.
template <class T>
static int lq_pullback_run(cudaStream_t st, int64_t m, int64_t n, int full, T* dA, int64_t ldda,
                           const T* L, int64_t ldl, const T* Q, int64_t ldq, const T* dL,
                           int64_t lddl, const T* dQ, int64_t lddq, double rank_atol,
                           double gauge_atol, int precision, Arena& ar, mak_info* info) {
  const int64_t k = m < n ? m : n;
  const int64_t qr_ = (full && n > m) ? n : k;  // rows of Q, columns of L
  const int64_t lq = qr_ > 0 ? qr_ : 1;
  const int64_t ln = n > 0 ? n : 1;
  T* Qt = ar.take<T>((size_t)n * qr_ + 1);
  T* Rt = ar.take<T>((size_t)qr_ * m + 1);
  T* dQt = dQ ? ar.take<T>((size_t)n * qr_ + 1) : nullptr;
  T* dRt = dL ? ar.take<T>((size_t)qr_ * m + 1) : nullptr;
  T* dB = ar.take<T>((size_t)n * m + 1);
  size_t inner = 0;
  {
    Arena meas(nullptr, 0);
    qr_pullback_run<T>(st, n, m, full, nullptr, ln, nullptr, ln, nullptr, lq, nullptr, ln,
                       nullptr, lq, rank_atol, gauge_atol, precision, meas, nullptr);
    inner = meas.off + 256;
  }
  char* sub = ar.take<char>(inner);
  if (ar.base == nullptr) return 0;
  if (!ar.ok()) return MAK_ERR_WORKSPACE;
  MAK_TRY(ctranspose<T>(st, qr_, n, Q, ldq, Qt, ln));
  MAK_TRY(ctranspose<T>(st, m, qr_, L, ldl, Rt, lq));
  if (dQ) MAK_TRY(ctranspose<T>(st, qr_, n, dQ, lddq, dQt, ln));
  if (dL) MAK_TRY(ctranspose<T>(st, m, qr_, dL, lddl, dRt, lq));
  if (n * m > 0) MAK_CUDA_TRY(cudaMemsetAsync(dB, 0, (size_t)n * m * sizeof(T), st));
  Arena a2(sub, inner);
  MAK_TRY(qr_pullback_run<T>(st, n, m, full, dB, ln, Qt, ln, Rt, lq, dQt, ln, dRt, lq, rank_atol,
                             gauge_atol, precision, a2, info));
  return ctranspose<T>(st, n, m, dB, ln, dA, ldda, true);
}

// lq_null_pullback! (reference src/pullbacks/lq.jl:133-145): the conjugate
// transpose of qr_null_pullback! of A^H at N = Nh^H with dN = dNh^H
// (X = L^{-H} Q dNh^H, dA -= X Nh; the gauge ||antiherm(Nh dNh^H)||_F).
template <class T>
static int lq_null_pullback_run(cudaStream_t st, int64_t m, int64_t n, T* dA, int64_t ldda,
                                const T* A, int64_t lda, const T* Nh, int64_t ldnh,
                                const T* dNh, int64_t lddnh, double gauge_atol, int precision,
                                Arena& ar, mak_info* info) {
  const int64_t k = m < n ? m : n;
  const int64_t nr = n - k;
  const int64_t ln = n > 0 ? n : 1;
  T* At = ar.take<T>((size_t)n * m + 1);
  T* Nt = ar.take<T>((size_t)n * nr + 1);
  T* dNt = ar.take<T>((size_t)n * nr + 1);
  T* dB = ar.take<T>((size_t)n * m + 1);
  size_t inner = 0;
  {
    Arena meas(nullptr, 0);
    qr_null_pullback_run<T>(st, n, m, nullptr, ln, nullptr, ln, nullptr, ln, nullptr, ln,
                            gauge_atol, precision, meas, nullptr);
    inner = meas.off + 256;
  }
  char* sub = ar.take<char>(inner);
  if (ar.base == nullptr) return 0;
  if (!ar.ok()) return MAK_ERR_WORKSPACE;
  MAK_TRY(ctranspose<T>(st, m, n, A, lda, At, ln));
  MAK_TRY(ctranspose<T>(st, nr, n, Nh, ldnh, Nt, ln));
  if (dNh) MAK_TRY(ctranspose<T>(st, nr, n, dNh, lddnh, dNt, ln));
  if (n * m > 0) MAK_CUDA_TRY(cudaMemsetAsync(dB, 0, (size_t)n * m * sizeof(T), st));
  Arena a2(sub, inner);
  MAK_TRY(qr_null_pullback_run<T>(st, n, m, dB, ln, At, ln, Nt, ln, dNh ? dNt : nullptr, ln,
                                  gauge_atol, precision, a2, info));
  return ctranspose<T>(st, n, m, dB, ln, dA, ldda, true);
}

template <class T>
static int qr_null_pullback_entry(int64_t m, int64_t n, void* dAv, int64_t ldda, const void* Av,
                                  int64_t lda, const void* Nv, int64_t ldn, const void* dNv,
                                  int64_t lddn, const mak_pullback_opts* opts, void* work,
                                  size_t work_bytes, mak_info* info, mak_stream_t stream) {
  const int64_t k = m < n ? m : n;
  const int64_t nc = m - k;
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (dAv == nullptr && m * n > 0) return -3;
  if (ldda < (m > 1 ? m : 1)) return -4;
  if (Av == nullptr && m * n > 0) return -5;
  if (lda < (m > 1 ? m : 1)) return -6;
  if (Nv == nullptr && m * nc > 0) return -7;
  if (ldn < (m > 1 ? m : 1)) return -8;
  if (dNv && lddn < (m > 1 ? m : 1)) return -10;
  mak_pullback_opts o{-1.0, -1.0, MAK_PREC_NATIVE, 0};
  if (opts) o = *opts;
  if (o.precision != MAK_PREC_NATIVE && o.precision != MAK_PREC_MIXED) return -11;
  if (info == nullptr) return -14;
  cudaStream_t st = (cudaStream_t)stream;
  {
    Arena meas(nullptr, 0);
    qr_null_pullback_run<T>(st, m, n, nullptr, ldda, nullptr, lda, nullptr, ldn, nullptr, lddn,
                            o.gauge_atol, o.precision, meas, nullptr);
    if (meas.off > work_bytes) return -13;
  }
  MAK_TRY(info_reset(st, info));
  Arena ar(work, work_bytes);
  return qr_null_pullback_run<T>(st, m, n, (T*)dAv, ldda, (const T*)Av, lda, (const T*)Nv, ldn,
                                 (const T*)dNv, lddn, o.gauge_atol, o.precision, ar, info);
}

template <class T>
static int lq_pullback_entry(int64_t m, int64_t n, int full, void* dAv, int64_t ldda,
                             const void* Lv, int64_t ldl, const void* Qv, int64_t ldq,
                             const void* dLv, int64_t lddl, const void* dQv, int64_t lddq,
                             const mak_pullback_opts* opts, void* work, size_t work_bytes,
                             mak_info* info, mak_stream_t stream) {
  const int64_t k = m < n ? m : n;
  const int64_t qr_ = (full && n > m) ? n : k;
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (dAv == nullptr && m * n > 0) return -4;
  if (ldda < (m > 1 ? m : 1)) return -5;
  if (Lv == nullptr && m * qr_ > 0) return -6;
  if (ldl < (m > 1 ? m : 1)) return -7;
  if (Qv == nullptr && qr_ * n > 0) return -8;
  if (ldq < (qr_ > 1 ? qr_ : 1)) return -9;
  if (dLv && lddl < (m > 1 ? m : 1)) return -11;
  if (dQv && lddq < (qr_ > 1 ? qr_ : 1)) return -13;
  mak_pullback_opts o{-1.0, -1.0, MAK_PREC_NATIVE, 0};
  if (opts) o = *opts;
  if (o.precision != MAK_PREC_NATIVE && o.precision != MAK_PREC_MIXED) return -14;
  if (info == nullptr) return -17;
  cudaStream_t st = (cudaStream_t)stream;
  {
    Arena meas(nullptr, 0);
    lq_pullback_run<T>(st, m, n, full, nullptr, ldda, nullptr, ldl, nullptr, ldq,
                       (const T*)dLv, lddl, (const T*)dQv, lddq, o.rank_atol, o.gauge_atol,
                       o.precision, meas, nullptr);
    if (meas.off > work_bytes) return -16;
  }
  MAK_TRY(info_reset(st, info));
  Arena ar(work, work_bytes);
  return lq_pullback_run<T>(st, m, n, full, (T*)dAv, ldda, (const T*)Lv, ldl, (const T*)Qv, ldq,
                            (const T*)dLv, lddl, (const T*)dQv, lddq, o.rank_atol, o.gauge_atol,
                            o.precision, ar, info);
}

template <class T>
static int lq_null_pullback_entry(int64_t m, int64_t n, void* dAv, int64_t ldda, const void* Av,
                                  int64_t lda, const void* Nhv, int64_t ldnh, const void* dNhv,
                                  int64_t lddnh, const mak_pullback_opts* opts, void* work,
                                  size_t work_bytes, mak_info* info, mak_stream_t stream) {
  const int64_t k = m < n ? m : n;
  const int64_t nr = n - k;
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (dAv == nullptr && m * n > 0) return -3;
  if (ldda < (m > 1 ? m : 1)) return -4;
  if (Av == nullptr && m * n > 0) return -5;
  if (lda < (m > 1 ? m : 1)) return -6;
  if (Nhv == nullptr && nr * n > 0) return -7;
  if (ldnh < (nr > 1 ? nr : 1)) return -8;
  if (dNhv && lddnh < (nr > 1 ? nr : 1)) return -10;
  mak_pullback_opts o{-1.0, -1.0, MAK_PREC_NATIVE, 0};
  if (opts) o = *opts;
  if (o.precision != MAK_PREC_NATIVE && o.precision != MAK_PREC_MIXED) return -11;
  if (info == nullptr) return -14;
  cudaStream_t st = (cudaStream_t)stream;
  {
    Arena meas(nullptr, 0);
    lq_null_pullback_run<T>(st, m, n, nullptr, ldda, nullptr, lda, nullptr, ldnh, nullptr, lddnh,
                            o.gauge_atol, o.precision, meas, nullptr);
    if (meas.off > work_bytes) return -13;
  }
  MAK_TRY(info_reset(st, info));
  Arena ar(work, work_bytes);
  return lq_null_pullback_run<T>(st, m, n, (T*)dAv, ldda, (const T*)Av, lda, (const T*)Nhv, ldnh,
                                 (const T*)dNhv, lddnh, o.gauge_atol, o.precision, ar, info);
}

template <class T>
static size_t qr_null_pb_ws(int64_t m, int64_t n, int prec) {
  Arena meas(nullptr, 0);
  qr_null_pullback_run<T>(0, m, n, nullptr, m, nullptr, m, nullptr, m, nullptr, m, -1.0, prec,
                          meas, nullptr);
  return meas.off + 256;
}
template <class T>
static size_t lq_pb_ws(int64_t m, int64_t n, int full, int prec) {
  Arena meas(nullptr, 0);
  T dummy;
  // with both cotangents present (the larger workspace)
  lq_pullback_run<T>(0, m, n, full, nullptr, m, nullptr, m, nullptr, n, &dummy, m, &dummy, n,
                     -1.0, -1.0, prec, meas, nullptr);
  return meas.off + 256;
}
template <class T>
static size_t lq_null_pb_ws(int64_t m, int64_t n, int prec) {
  Arena meas(nullptr, 0);
  lq_null_pullback_run<T>(0, m, n, nullptr, m, nullptr, m, nullptr, n, nullptr, n, -1.0, prec,
                          meas, nullptr);
  return meas.off + 256;
}

template <class T>
static size_t qr_pb_ws(int64_t m, int64_t n, int full, int prec) {
  Arena meas(nullptr, 0);
  qr_pullback_run<T>(0, m, n, full, nullptr, m, nullptr, m, nullptr, m, nullptr, m, nullptr, m,
                     -1.0, -1.0, prec, meas, nullptr);
  return meas.off + 256;
}
template <class T>
static size_t polar_pb_ws(int64_t m, int64_t n, int prec) {
  Arena meas(nullptr, 0);
  polar_pullback_run<T>(0, m, n, nullptr, m, nullptr, m, nullptr, n, nullptr, m, nullptr, n,
                        SIGN_MAXITER, prec, meas, nullptr);
  return meas.off + 256;
}

}  // namespace mak

using namespace mak;

extern "C" {

int mak_qr_pullback_workspace(int dtype, int64_t m, int64_t n, int full, int precision,
                              size_t* bytes) {
  if (bytes == nullptr) return -6;
  if (m < 0) return -2;
  if (n < 0) return -3;
  switch (dtype) {
    case MAK_F64: *bytes = qr_pb_ws<double>(m, n, full, precision); break;
    case MAK_C64: *bytes = qr_pb_ws<zcomplex>(m, n, full, precision); break;
    case MAK_F32: *bytes = qr_pb_ws<float>(m, n, full, precision); break;
    case MAK_C32: *bytes = qr_pb_ws<ccomplex>(m, n, full, precision); break;
    default: return -1;
  }
  return 0;
}

int mak_left_polar_pullback_workspace(int dtype, int64_t m, int64_t n, int precision,
                                      size_t* bytes) {
  if (bytes == nullptr) return -5;
  if (m < 0) return -2;
  if (n < 0 || n > m) return -3;
  switch (dtype) {
    case MAK_F64: *bytes = polar_pb_ws<double>(m, n, precision); break;
    case MAK_C64: *bytes = polar_pb_ws<zcomplex>(m, n, precision); break;
    case MAK_F32: *bytes = polar_pb_ws<float>(m, n, precision); break;
    case MAK_C32: *bytes = polar_pb_ws<ccomplex>(m, n, precision); break;
    default: return -1;
  }
  return 0;
}

#define MAK_QRPB(NAME, T, PT)                                                                   \
  int NAME(int64_t m, int64_t n, int full, PT* dA, int64_t ldda, const PT* Q, int64_t ldq,      \
           const PT* R, int64_t ldr, const PT* dQ, int64_t lddq, const PT* dR, int64_t lddr,    \
           const mak_pullback_opts* opts, void* work, size_t work_bytes, mak_info* info,        \
           mak_stream_t stream) {                                                               \
    return qr_pullback_entry<T>(m, n, full, dA, ldda, Q, ldq, R, ldr, dQ, lddq, dR, lddr, opts, \
                                work, work_bytes, info, stream);                               \
  }
MAK_QRPB(mak_qr_pullback_d, double, double)
MAK_QRPB(mak_qr_pullback_z, zcomplex, void)
MAK_QRPB(mak_qr_pullback_s, float, float)
MAK_QRPB(mak_qr_pullback_c, ccomplex, void)

#define MAK_POLPB(NAME, T, PT)                                                                  \
  int NAME(int64_t m, int64_t n, PT* dA, int64_t ldda, const PT* W, int64_t ldw, const PT* P,   \
           int64_t ldp, const PT* dW, int64_t lddw, const PT* dP, int64_t lddp,                 \
           const mak_pullback_opts* opts, void* work, size_t work_bytes, mak_info* info,        \
           mak_stream_t stream) {                                                               \
    return polar_pullback_entry<T>(m, n, dA, ldda, W, ldw, P, ldp, dW, lddw, dP, lddp, opts,    \
                                   work, work_bytes, info, stream);                            \
  }
MAK_POLPB(mak_left_polar_pullback_d, double, double)
MAK_POLPB(mak_left_polar_pullback_z, zcomplex, void)
MAK_POLPB(mak_left_polar_pullback_s, float, float)
MAK_POLPB(mak_left_polar_pullback_c, ccomplex, void)

int mak_left_polar_pushforward_workspace(int dtype, int64_t m, int64_t n, int precision,
                                         size_t* bytes) {
  if (bytes == nullptr) return -5;
  if (m < 0) return -2;
  if (n < 0 || n > m) return -3;
  switch (dtype) {
    case MAK_F64: *bytes = polar_pf_ws<double>(m, n, precision); break;
    case MAK_C64: *bytes = polar_pf_ws<zcomplex>(m, n, precision); break;
    case MAK_F32: *bytes = polar_pf_ws<float>(m, n, precision); break;
    case MAK_C32: *bytes = polar_pf_ws<ccomplex>(m, n, precision); break;
    default: return -1;
  }
  return 0;
}

int mak_right_polar_pullback_workspace(int dtype, int64_t m, int64_t n, int precision,
                                       size_t* bytes) {
  if (bytes == nullptr) return -5;
  if (m < 0) return -2;
  if (n < m) return -3;
  switch (dtype) {
    case MAK_F64: *bytes = rpolar_pb_ws<double>(m, n, precision); break;
    case MAK_C64: *bytes = rpolar_pb_ws<zcomplex>(m, n, precision); break;
    case MAK_F32: *bytes = rpolar_pb_ws<float>(m, n, precision); break;
    case MAK_C32: *bytes = rpolar_pb_ws<ccomplex>(m, n, precision); break;
    default: return -1;
  }
  return 0;
}

int mak_right_polar_pushforward_workspace(int dtype, int64_t m, int64_t n, int precision,
                                          size_t* bytes) {
  if (bytes == nullptr) return -5;
  if (m < 0) return -2;
  if (n < m) return -3;
  switch (dtype) {
    case MAK_F64: *bytes = rpolar_pf_ws<double>(m, n, precision); break;
    case MAK_C64: *bytes = rpolar_pf_ws<zcomplex>(m, n, precision); break;
    case MAK_F32: *bytes = rpolar_pf_ws<float>(m, n, precision); break;
    case MAK_C32: *bytes = rpolar_pf_ws<ccomplex>(m, n, precision); break;
    default: return -1;
  }
  return 0;
}

#define MAK_RPOLPF(NAME, T, PT)                                                                 \
  int NAME(int64_t m, int64_t n, const PT* dA, int64_t ldda, const PT* P, int64_t ldp,          \
           const PT* Wh, int64_t ldwh, PT* dP, int64_t lddp, PT* dWh, int64_t lddwh,            \
           const mak_pullback_opts* opts, void* work, size_t work_bytes, mak_info* info,        \
           mak_stream_t stream) {                                                               \
    return right_polar_pushforward_entry<T>(m, n, dA, ldda, P, ldp, Wh, ldwh, dP, lddp, dWh,    \
                                            lddwh, opts, work, work_bytes, info, stream);       \
  }
MAK_RPOLPF(mak_right_polar_pushforward_d, double, double)
MAK_RPOLPF(mak_right_polar_pushforward_z, zcomplex, void)
MAK_RPOLPF(mak_right_polar_pushforward_s, float, float)
MAK_RPOLPF(mak_right_polar_pushforward_c, ccomplex, void)

int mak_qr_null_pullback_workspace(int dtype, int64_t m, int64_t n, int precision,
                                   size_t* bytes) {
  if (bytes == nullptr) return -5;
  if (m < 0) return -2;
  if (n < 0) return -3;
  switch (dtype) {
    case MAK_F64: *bytes = qr_null_pb_ws<double>(m, n, precision); break;
    case MAK_C64: *bytes = qr_null_pb_ws<zcomplex>(m, n, precision); break;
    case MAK_F32: *bytes = qr_null_pb_ws<float>(m, n, precision); break;
    case MAK_C32: *bytes = qr_null_pb_ws<ccomplex>(m, n, precision); break;
    default: return -1;
  }
  return 0;
}

int mak_lq_pullback_workspace(int dtype, int64_t m, int64_t n, int full, int precision,
                              size_t* bytes) {
  if (bytes == nullptr) return -6;
  if (m < 0) return -2;
  if (n < 0) return -3;
  switch (dtype) {
    case MAK_F64: *bytes = lq_pb_ws<double>(m, n, full, precision); break;
    case MAK_C64: *bytes = lq_pb_ws<zcomplex>(m, n, full, precision); break;
    case MAK_F32: *bytes = lq_pb_ws<float>(m, n, full, precision); break;
    case MAK_C32: *bytes = lq_pb_ws<ccomplex>(m, n, full, precision); break;
    default: return -1;
  }
  return 0;
}

int mak_lq_null_pullback_workspace(int dtype, int64_t m, int64_t n, int precision,
                                   size_t* bytes) {
  if (bytes == nullptr) return -5;
  if (m < 0) return -2;
  if (n < 0) return -3;
  switch (dtype) {
    case MAK_F64: *bytes = lq_null_pb_ws<double>(m, n, precision); break;
    case MAK_C64: *bytes = lq_null_pb_ws<zcomplex>(m, n, precision); break;
    case MAK_F32: *bytes = lq_null_pb_ws<float>(m, n, precision); break;
    case MAK_C32: *bytes = lq_null_pb_ws<ccomplex>(m, n, precision); break;
    default: return -1;
  }
  return 0;
}

#define MAK_NULLPB(NAME, FN, T, PT)                                                             \
  int NAME(int64_t m, int64_t n, PT* dA, int64_t ldda, const PT* A, int64_t lda, const PT* N,   \
           int64_t ldn, const PT* dN, int64_t lddn, const mak_pullback_opts* opts, void* work,  \
           size_t work_bytes, mak_info* info, mak_stream_t stream) {                            \
    return FN<T>(m, n, dA, ldda, A, lda, N, ldn, dN, lddn, opts, work, work_bytes, info,        \
                 stream);                                                                       \
  }
MAK_NULLPB(mak_qr_null_pullback_d, qr_null_pullback_entry, double, double)
MAK_NULLPB(mak_qr_null_pullback_z, qr_null_pullback_entry, zcomplex, void)
MAK_NULLPB(mak_qr_null_pullback_s, qr_null_pullback_entry, float, float)
MAK_NULLPB(mak_qr_null_pullback_c, qr_null_pullback_entry, ccomplex, void)
MAK_NULLPB(mak_lq_null_pullback_d, lq_null_pullback_entry, double, double)
MAK_NULLPB(mak_lq_null_pullback_z, lq_null_pullback_entry, zcomplex, void)
MAK_NULLPB(mak_lq_null_pullback_s, lq_null_pullback_entry, float, float)
MAK_NULLPB(mak_lq_null_pullback_c, lq_null_pullback_entry, ccomplex, void)

#define MAK_LQPB(NAME, T, PT)                                                                   \
  int NAME(int64_t m, int64_t n, int full, PT* dA, int64_t ldda, const PT* L, int64_t ldl,      \
           const PT* Q, int64_t ldq, const PT* dL, int64_t lddl, const PT* dQ, int64_t lddq,    \
           const mak_pullback_opts* opts, void* work, size_t work_bytes, mak_info* info,        \
           mak_stream_t stream) {                                                               \
    return lq_pullback_entry<T>(m, n, full, dA, ldda, L, ldl, Q, ldq, dL, lddl, dQ, lddq, opts, \
                                work, work_bytes, info, stream);                                \
  }
MAK_LQPB(mak_lq_pullback_d, double, double)
MAK_LQPB(mak_lq_pullback_z, zcomplex, void)
MAK_LQPB(mak_lq_pullback_s, float, float)
MAK_LQPB(mak_lq_pullback_c, ccomplex, void)

#define MAK_POLPF(NAME, T, PT)                                                                  \
  int NAME(int64_t m, int64_t n, const PT* dA, int64_t ldda, const PT* W, int64_t ldw,          \
           const PT* P, int64_t ldp, PT* dW, int64_t lddw, PT* dP, int64_t lddp,                \
           const mak_pullback_opts* opts, void* work, size_t work_bytes, mak_info* info,        \
           mak_stream_t stream) {                                                               \
    return polar_pushforward_entry<T>(m, n, dA, ldda, W, ldw, P, ldp, dW, lddw, dP, lddp, opts, \
                                      work, work_bytes, info, stream);                         \
  }
MAK_POLPF(mak_left_polar_pushforward_d, double, double)
MAK_POLPF(mak_left_polar_pushforward_z, zcomplex, void)
MAK_POLPF(mak_left_polar_pushforward_s, float, float)
MAK_POLPF(mak_left_polar_pushforward_c, ccomplex, void)

#define MAK_RPOLPB(NAME, T, PT)                                                                 \
  int NAME(int64_t m, int64_t n, PT* dA, int64_t ldda, const PT* P, int64_t ldp, const PT* Wh,  \
           int64_t ldwh, const PT* dP, int64_t lddp, const PT* dWh, int64_t lddwh,              \
           const mak_pullback_opts* opts, void* work, size_t work_bytes, mak_info* info,        \
           mak_stream_t stream) {                                                               \
    return right_polar_pullback_entry<T>(m, n, dA, ldda, P, ldp, Wh, ldwh, dP, lddp, dWh,       \
                                         lddwh, opts, work, work_bytes, info, stream);          \
  }
MAK_RPOLPB(mak_right_polar_pullback_d, double, double)
MAK_RPOLPB(mak_right_polar_pullback_z, zcomplex, void)
MAK_RPOLPB(mak_right_polar_pullback_s, float, float)
MAK_RPOLPB(mak_right_polar_pullback_c, ccomplex, void)

}  // extern "C"
