// Householder QR of small blocks, one CTA per block, from a work list.
//
// For a block whose m x n elements fit one CTA's shared memory, the batched
// driver's per-block chain of launches (panels, block updates, Q formation:
// qr_householder!, src/implementations/qr.jl:132-188, once per block) is
// replaced by a single persistent launch that walks a list of block
// descriptors (mak_batch_item): CTA b takes items b, b + gridDim.x, ...
// and for each
//   1. loads the block into shared memory,
//   2. factors it column by column (LAPACK geqr2 order; the reflector
//      scalars come from the same larfg helpers as the multi-CTA panel, so
//      beta is real and R's diagonal carries its sign),
//   3. writes R with the positive gauge (rows scaled by conj(s_i), s =
//      sign_safe(diag R), src/common/gauge.jl:16-25),
//   4. forms Q in place over the reflectors (org2r order: H_{k-1} first on
//      [I_k; 0], the identity structure leaves columns < j untouched at
//      step j) and writes Q diag(s).
// The list lives either in device memory (mak_batched_qr_compact_device:
// a caller-built list, e.g. produced by a previous kernel) or in the
// launch's parameters (the batched driver's small items, copied by value
// into a captured CUDA graph).  Items that do not fit report
// MAK_ERR_UNSUPPORTED in their record.
#include "householder.cuh"
#include "internal.h"

namespace mak {

constexpr int SMALL_THREADS = 256;
constexpr int SMALL_LIST_MAX = 400;  // items per parameter-list launch (72 + 4 bytes each)

struct SmallList {
  int count;
  int pad;
  mak_batch_item items[SMALL_LIST_MAX];
  int idx[SMALL_LIST_MAX];  // each item's position in the caller's list (its mak_info)
};
static_assert(sizeof(SmallList) <= 32000, "kernel parameter space");

// shared scratch of one CTA (raw bytes: the element type varies per item)
struct SmallScratch {
  double red_r[32];
  unsigned long long red_k[32];
  double sc_r[2];
  int sc_flag;
  alignas(16) unsigned char sc[3 * 16];  // beta, tau, scal
};

__host__ __device__ size_t small_qr_bytes(int dtype, int64_t m, int64_t n) {
  const size_t es = (dtype == MAK_F64 || dtype == MAK_C32) ? 8 : (dtype == MAK_C64 ? 16 : 4);
  const int64_t k = m < n ? m : n;
  return (size_t)(m * n + 2 * k) * es;  // the block, tau and the gauge signs
}

template <class T>
__device__ void small_qr_item(const mak_batch_item& it, int positive, mak_info* info,
                              unsigned char* dyn, int cap_bytes, SmallScratch& sh) {
  using R = real_t<T>;
  using NK = NormKey<R>;
  using Key = typename NK::K;
  const int64_t m64 = it.m, n64 = it.n;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  const int bd = blockDim.x;
  if (tid == 0) {
    info->status = 0;
    info->iterations = 0;
    info->rank = 0;
    info->converged = 0;
    info->residual = 0.0;
    info->gauge = 0.0;
    info->gauge_atol = 0.0;
    info->singular = 0;
    info->pad = 0;
  }
  if (m64 < 0 || n64 < 0 || small_qr_bytes(it.dtype, m64, n64) > (size_t)cap_bytes) {
    if (tid == 0) info->status = MAK_ERR_UNSUPPORTED;
    return;
  }
  const int m = (int)m64, n = (int)n64, k = m < n ? m : n;
  if (k == 0) return;
  const T* A = (const T*)it.A;
  T* S = reinterpret_cast<T*>(dyn);  // m x n, ld m
  T* taus = S + (int64_t)m * n;      // k
  T* sgn = taus + k;                 // k
  for (int c = 0; c < n; c++)
    for (int r = tid; r < m; r += bd) S[r + c * m] = A[r + (int64_t)c * it.lda];
  __syncthreads();

  // ---- factorization: one reflector per column
  R* red_r = reinterpret_cast<R*>(sh.red_r);
  Key* red_k = reinterpret_cast<Key*>(sh.red_k);
  T* sc = reinterpret_cast<T*>(sh.sc);
  for (int j = 0; j < k; j++) {
    T* col = S + j * m;
    // sum of squares and largest magnitude of x = column j below the diagonal
    R ss = R(0);
    Key mk = 0;
    for (int r = j + 1 + tid; r < m; r += bd) {
      const T x = col[r];
      ss = sq_add(ss, x);
      const Key q = mag_key(x);
      mk = q > mk ? q : mk;
    }
    ss = warp_sum(ss);
    mk = warp_max_key(mk);
    if (lane == 0) {
      red_r[wid] = ss;
      red_k[wid] = mk;
    }
    __syncthreads();
    if (tid == 0) {
      R s2 = R(0);
      Key m2 = 0;
      for (int w = 0; w < nw; w++) {
        s2 += red_r[w];
        m2 = red_k[w] > m2 ? red_k[w] : m2;
      }
      sh.sc_r[0] = (double)s2;
      sh.sc_r[1] = (double)NK::val(m2);
      sh.sc_flag = norm_needs_rescale<R>(m2);
    }
    __syncthreads();
    R xnorm = R(0);
    const bool rescale = sh.sc_flag != 0;
    if (rescale) {
      // rare: the squares would overflow or underflow; sum them scaled by
      // 2^-e, e the exponent of the largest magnitude (clamped)
      int e = 0;
      frexp((R)sh.sc_r[1], &e);
      e = e > 1000 ? 1000 : (e < -1000 ? -1000 : e);
      const R scale = ldexp(R(1), -e);
      R s3 = R(0);
      for (int r = j + 1 + tid; r < m; r += bd) ssq_scaled_add(s3, col[r], scale);
      s3 = block_sum(s3, red_r);
      xnorm = sqrt(s3) * ldexp(R(1), e);
    }
    if (tid == 0) {
      T beta, tau, scal;
      if (rescale) larfg_scalars(col[j], xnorm, beta, tau, scal);
      else larfg_scalars_ssq(col[j], (R)sh.sc_r[0], (R)sh.sc_r[1], beta, tau, scal);
      sc[0] = beta;
      sc[1] = tau;
      sc[2] = scal;
      taus[j] = tau;
    }
    __syncthreads();
    const T beta = sc[0], tau = sc[1], scal = sc[2];
    for (int r = j + 1 + tid; r < m; r += bd) col[r] = col[r] * scal;
    __syncthreads();
    // H_j^H on the columns to the right: w_c = A[j,c] + sum_{r>j} conj(v_r)
    // A[r,c], A[:,c] -= v conj(tau) w_c (v_j = 1); a warp per column
    for (int c = j + 1 + wid; c < n; c += nw) {
      T* pc = S + c * m;
      const T ajc = pc[j];
      T acc = zero_<T>();
      for (int r = j + 1 + lane; r < m; r += 32) acc = fma_(conj_(col[r]), pc[r], acc);
      acc = warp_sum(acc);
      const T f = conj_(tau) * (ajc + acc);
      __syncwarp();
      if (lane == 0) pc[j] = ajc - f;
      for (int r = j + 1 + lane; r < m; r += 32) pc[r] = fma_(-col[r], f, pc[r]);
    }
    if (tid == 0) col[j] = beta;
    __syncthreads();
  }

  // ---- R with the gauge: R[i, c] = conj(s_i) A[i, c] (i <= c), 0 below
  for (int i = tid; i < k; i += bd) sgn[i] = positive ? sign_safe_(S[i + i * m]) : one_<T>();
  __syncthreads();
  if (it.R != nullptr) {
    T* Rout = (T*)it.R;
    for (int c = 0; c < n; c++)
      for (int i = tid; i < k; i += bd)
        Rout[i + (int64_t)c * it.ldr] = (i <= c) ? conj_(sgn[i]) * S[i + c * m] : zero_<T>();
  }
  __syncthreads();

  // ---- Q = H_0 ... H_{k-1} [I_k; 0], formed in place over the reflectors
  for (int j = k - 1; j >= 0; j--) {
    T* col = S + j * m;
    const T tau = taus[j];
    // H_j on the columns c in (j, k): rows >= j (rows < j are zero there)
    for (int c = j + 1 + wid; c < k; c += nw) {
      T* pc = S + c * m;
      const T qj = pc[j];
      T acc = zero_<T>();
      for (int r = j + 1 + lane; r < m; r += 32) acc = fma_(conj_(col[r]), pc[r], acc);
      acc = warp_sum(acc);
      const T f = tau * (qj + acc);
      __syncwarp();
      if (lane == 0) pc[j] = qj - f;
      for (int r = j + 1 + lane; r < m; r += 32) pc[r] = fma_(-col[r], f, pc[r]);
    }
    __syncthreads();
    // column j of Q: e_j - tau v
    for (int r = tid; r < m; r += bd) {
      T q;
      if (r < j) q = zero_<T>();
      else if (r == j) q = one_<T>() - tau;
      else q = -(tau * col[r]);
      col[r] = q;
    }
    __syncthreads();
  }
  T* Qout = (T*)it.Q;
  for (int c = 0; c < k; c++)
    for (int r = tid; r < m; r += bd) Qout[r + (int64_t)c * it.ldq] = S[r + c * m] * sgn[c];
}

// ---------------------------------------------------------------- polar --
// left_polar! (PolarNewton) of a small block in one CTA, the reference's
// left_polar_newton! (src/implementations/polar.jl:128-166): for m > n the
// Newton iteration runs on R of A = QR (the QR above, no gauge: the polar
// factor does not depend on it), else on A itself.  Each step inverts the
// iterate by Gauss-Jordan with partial pivoting in shared memory, scales by
// g = (||X^-1||_F / ||X||_F)^(1/2) and averages, X <- (g X + X^-H / g) / 2,
// with conv = max |X^-H / g - g X|; the loop takes at most maxiter steps
// and stops once conv <= tol (or is not a number), the first step always
// (the same rule as the reference's host loop).  P = herm(X^H R) (R = A for
// m = n) is formed before Q, then W = Q X.
__host__ __device__ size_t small_polar_bytes(int dtype, int64_t m, int64_t n) {
  const size_t es = (dtype == MAK_F64 || dtype == MAK_C32) ? 8 : (dtype == MAK_C64 ? 16 : 4);
  // A / reflectors (m n), X and Y (n^2 each), tau and a pivot column (n
  // each), the pivot rows (n ints)
  return (size_t)(m * n + 2 * n * n + 2 * n) * es + (size_t)n * sizeof(int);
}

template <class T>
__device__ void small_polar_item(const mak_batch_item& it, int maxiter, double tol,
                                 mak_info* info, unsigned char* dyn, int cap_bytes,
                                 SmallScratch& sh) {
  using R = real_t<T>;
  const int64_t m64 = it.m, n64 = it.n;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  const int bd = blockDim.x;
  if (tid == 0) {
    info->status = 0;
    info->iterations = 0;
    info->rank = 0;
    info->converged = 0;
    info->residual = 0.0;
    info->gauge = 0.0;
    info->gauge_atol = 0.0;
    info->singular = 0;
    info->pad = 0;
  }
  if (m64 < n64 || n64 < 0 || small_polar_bytes(it.dtype, m64, n64) > (size_t)cap_bytes) {
    if (tid == 0) info->status = MAK_ERR_UNSUPPORTED;
    return;
  }
  const int m = (int)m64, n = (int)n64;
  if (n == 0) {
    if (tid == 0) info->converged = 1;
    return;
  }
  T* Qb = reinterpret_cast<T*>(dyn);  // m x n: A, its reflectors, then Q
  T* X = Qb + (int64_t)m * n;         // n x n iterate, ld n
  T* Y = X + n * n;                   // n x n inverse, ld n
  T* taus = Y + n * n;                // n
  T* fcol = taus + n;                 // n: the pivot column during elimination
  int* piv = reinterpret_cast<int*>(fcol + n);
  const T* A = (const T*)it.A;
  for (int c = 0; c < n; c++)
    for (int r = tid; r < m; r += bd) Qb[r + c * m] = A[r + (int64_t)c * it.lda];
  __syncthreads();
  R* red_r = reinterpret_cast<R*>(sh.red_r);
  T* sc = reinterpret_cast<T*>(sh.sc);
  const bool qr = m > n;
  if (qr) {
    // Householder QR of the block (no gauge), R left in the upper triangle
    using NK = NormKey<R>;
    using Key = typename NK::K;
    Key* red_k = reinterpret_cast<Key*>(sh.red_k);
    for (int j = 0; j < n; j++) {
      T* col = Qb + j * m;
      R ss = R(0);
      Key mk = 0;
      for (int r = j + 1 + tid; r < m; r += bd) {
        const T x = col[r];
        ss = sq_add(ss, x);
        const Key q = mag_key(x);
        mk = q > mk ? q : mk;
      }
      ss = warp_sum(ss);
      mk = warp_max_key(mk);
      if (lane == 0) {
        red_r[wid] = ss;
        red_k[wid] = mk;
      }
      __syncthreads();
      if (tid == 0) {
        R s2 = R(0);
        Key m2 = 0;
        for (int w = 0; w < nw; w++) {
          s2 += red_r[w];
          m2 = red_k[w] > m2 ? red_k[w] : m2;
        }
        sh.sc_r[0] = (double)s2;
        sh.sc_r[1] = (double)NK::val(m2);
        sh.sc_flag = norm_needs_rescale<R>(m2);
      }
      __syncthreads();
      R xnorm = R(0);
      const bool rescale = sh.sc_flag != 0;
      if (rescale) {
        int e = 0;
        frexp((R)sh.sc_r[1], &e);
        e = e > 1000 ? 1000 : (e < -1000 ? -1000 : e);
        const R scale = ldexp(R(1), -e);
        R s3 = R(0);
        for (int r = j + 1 + tid; r < m; r += bd) ssq_scaled_add(s3, col[r], scale);
        s3 = block_sum(s3, red_r);
        xnorm = sqrt(s3) * ldexp(R(1), e);
      }
      if (tid == 0) {
        T beta, tau, scal;
        if (rescale) larfg_scalars(col[j], xnorm, beta, tau, scal);
        else larfg_scalars_ssq(col[j], (R)sh.sc_r[0], (R)sh.sc_r[1], beta, tau, scal);
        sc[0] = beta;
        sc[1] = tau;
        sc[2] = scal;
        taus[j] = tau;
      }
      __syncthreads();
      const T beta = sc[0], tau = sc[1], scal = sc[2];
      for (int r = j + 1 + tid; r < m; r += bd) col[r] = col[r] * scal;
      __syncthreads();
      for (int c = j + 1 + wid; c < n; c += nw) {
        T* pc = Qb + c * m;
        const T ajc = pc[j];
        T acc = zero_<T>();
        for (int r = j + 1 + lane; r < m; r += 32) acc = fma_(conj_(col[r]), pc[r], acc);
        acc = warp_sum(acc);
        const T f = conj_(tau) * (ajc + acc);
        __syncwarp();
        if (lane == 0) pc[j] = ajc - f;
        for (int r = j + 1 + lane; r < m; r += 32) pc[r] = fma_(-col[r], f, pc[r]);
      }
      if (tid == 0) col[j] = beta;
      __syncthreads();
    }
  }
  // X = R (upper triangle) or A
  for (int e = tid; e < n * n; e += bd) {
    const int i = e % n, j = e / n;
    X[e] = (!qr || i <= j) ? Qb[i + j * m] : zero_<T>();
  }
  __syncthreads();

  // ---- Newton iteration
  int steps = 0;
  bool singular = false;
  R conv = R(0);
  do {
    for (int e = tid; e < n * n; e += bd) Y[e] = X[e];
    __syncthreads();
    // Gauss-Jordan inverse of Y in place, partial (row) pivoting
    for (int k = 0; k < n; k++) {
      // pivot: the largest |Y[r, k]|, r >= k (ties: the first row)
      R best = R(-1);
      int bi = k;
      for (int r = k + tid; r < n; r += bd) {
        const R a = abs2_(Y[r + k * n]);
        if (a > best) {
          best = a;
          bi = r;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const R ob = shfl_xor_(best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      if (lane == 0) {
        red_r[wid] = best;
        sh.red_k[wid] = (unsigned long long)bi;
      }
      __syncthreads();
      if (tid == 0) {
        R b2 = red_r[0];
        int i2 = (int)sh.red_k[0];
        for (int w = 1; w < nw; w++) {
          const R bw = red_r[w];
          const int iw = (int)sh.red_k[w];
          if (bw > b2 || (bw == b2 && iw < i2)) {
            b2 = bw;
            i2 = iw;
          }
        }
        piv[k] = i2;
        sh.sc_flag = (b2 > R(0)) ? 0 : 1;
      }
      __syncthreads();
      if (sh.sc_flag) {  // an exactly singular iterate (the same in every thread)
        singular = true;
        break;
      }
      const int p = piv[k];
      if (p != k)
        for (int c = tid; c < n; c += bd) {
          const T t = Y[k + c * n];
          Y[k + c * n] = Y[p + c * n];
          Y[p + c * n] = t;
        }
      __syncthreads();
      const T d = inv_(Y[k + k * n]);
      for (int r = tid; r < n; r += bd) fcol[r] = Y[r + k * n];
      __syncthreads();
      for (int c = tid; c < n; c += bd) Y[k + c * n] = (c == k) ? d : Y[k + c * n] * d;
      __syncthreads();
      for (int e = tid; e < n * n; e += bd) {
        const int r = e % n, c = e / n;
        if (r == k) continue;
        Y[e] = (c == k) ? -(fcol[r] * d) : fma_(-fcol[r], Y[k + c * n], Y[e]);
      }
      __syncthreads();
    }
    if (singular) break;
    for (int k = n - 1; k >= 0; k--) {
      const int p = piv[k];
      if (p != k)
        for (int r = tid; r < n; r += bd) {
          const T t = Y[r + k * n];
          Y[r + k * n] = Y[r + p * n];
          Y[r + p * n] = t;
        }
      __syncthreads();
    }
    // g = (||Y||_F^2 / ||X||_F^2)^(1/4); X <- (g X + Y^H / g) / 2
    R nx = R(0), ny = R(0);
    for (int e = tid; e < n * n; e += bd) {
      nx += abs2_(X[e]);
      ny += abs2_(Y[e]);
    }
    nx = block_sum(nx, red_r);
    ny = block_sum(ny, red_r);
    const R g = sqrt(sqrt(ny / nx)), ginv = R(1) / g;
    R dmax = R(0);
    for (int e = tid; e < n * n; e += bd) {
      const int i = e % n, j = e / n;
      const T yh = conj_(Y[j + i * n]) * ginv;
      const T gx = X[e] * g;
      dmax = fmax(dmax, abs_(yh - gx));
      X[e] = (gx + yh) * R(0.5);
    }
    conv = block_max(dmax, red_r);
    steps++;
    __syncthreads();
  } while (steps < maxiter && conv > (R)tol);

  if (tid == 0) {
    info->iterations = steps;
    info->residual = (double)conv;
    info->converged = (!singular && conv <= (R)tol) ? 1 : 0;
    info->singular = singular ? 1 : 0;
  }
  // ---- P = herm(X^H R) (R = A when m = n), via Y
  if (it.R != nullptr) {
    for (int e = tid; e < n * n; e += bd) {
      const int i = e % n, j = e / n;
      T acc = zero_<T>();
      for (int l = 0; l < n; l++) {
        const T rl = (!qr || l <= j) ? Qb[l + j * m] : zero_<T>();
        acc = fma_(conj_(X[l + i * n]), rl, acc);
      }
      Y[e] = acc;
    }
    __syncthreads();
    T* P = (T*)it.R;
    for (int e = tid; e < n * n; e += bd) {
      const int i = e % n, j = e / n;
      P[i + (int64_t)j * it.ldr] = (Y[i + j * n] + conj_(Y[j + i * n])) * R(0.5);
    }
  }
  __syncthreads();
  // ---- W = Q X (m > n; Q formed in place over the reflectors) or X
  T* W = (T*)it.Q;
  if (qr) {
    for (int j = n - 1; j >= 0; j--) {
      T* col = Qb + j * m;
      const T tau = taus[j];
      for (int c = j + 1 + wid; c < n; c += nw) {
        T* pc = Qb + c * m;
        const T qj = pc[j];
        T acc = zero_<T>();
        for (int r = j + 1 + lane; r < m; r += 32) acc = fma_(conj_(col[r]), pc[r], acc);
        acc = warp_sum(acc);
        const T f = tau * (qj + acc);
        __syncwarp();
        if (lane == 0) pc[j] = qj - f;
        for (int r = j + 1 + lane; r < m; r += 32) pc[r] = fma_(-col[r], f, pc[r]);
      }
      __syncthreads();
      for (int r = tid; r < m; r += bd) {
        T q;
        if (r < j) q = zero_<T>();
        else if (r == j) q = one_<T>() - tau;
        else q = -(tau * col[r]);
        col[r] = q;
      }
      __syncthreads();
    }
    for (int c = 0; c < n; c++)
      for (int r = tid; r < m; r += bd) {
        T acc = zero_<T>();
        for (int l = 0; l < n; l++) acc = fma_(Qb[r + l * m], X[l + c * n], acc);
        W[r + (int64_t)c * it.ldq] = acc;
      }
  } else {
    for (int c = 0; c < n; c++)
      for (int r = tid; r < n; r += bd) W[r + (int64_t)c * it.ldq] = X[r + c * n];
  }
}

__device__ void small_polar_dispatch(const mak_batch_item& it, int maxiter, double tol,
                                     mak_info* info, unsigned char* dyn, int cap_bytes,
                                     SmallScratch& sh) {
  switch (it.dtype) {
    case MAK_F64: small_polar_item<double>(it, maxiter, tol, info, dyn, cap_bytes, sh); break;
    case MAK_C64: small_polar_item<zcomplex>(it, maxiter, tol, info, dyn, cap_bytes, sh); break;
    case MAK_F32: small_polar_item<float>(it, maxiter, tol, info, dyn, cap_bytes, sh); break;
    case MAK_C32: small_polar_item<ccomplex>(it, maxiter, tol, info, dyn, cap_bytes, sh); break;
    default:
      if (threadIdx.x == 0) info->status = MAK_ERR_UNSUPPORTED;
  }
  __syncthreads();
}

// tol per element type: the caller's value, or eps(real T)^(2/3)
__device__ __forceinline__ double small_polar_tol(int dtype, double tol) {
  if (tol > 0) return tol;
  return (dtype == MAK_F64 || dtype == MAK_C64) ? 3.6700562101601e-11 : 2.4214387e-5;
}

__global__ void __launch_bounds__(SMALL_THREADS)
small_polar_list_kernel(const __grid_constant__ SmallList L, int maxiter, double tol,
                        mak_info* infos, int cap_bytes) {
  extern __shared__ __align__(16) unsigned char small_dyn[];
  __shared__ SmallScratch sh;
  for (int q = blockIdx.x; q < L.count; q += gridDim.x)
    small_polar_dispatch(L.items[q], maxiter, small_polar_tol(L.items[q].dtype, tol),
                         infos + L.idx[q], small_dyn, cap_bytes, sh);
}

__global__ void __launch_bounds__(SMALL_THREADS)
small_polar_device_kernel(const mak_batch_item* items, int count, int maxiter, double tol,
                          mak_info* infos, int cap_bytes) {
  extern __shared__ __align__(16) unsigned char small_dyn[];
  __shared__ SmallScratch sh;
  for (int q = blockIdx.x; q < count; q += gridDim.x)
    small_polar_dispatch(items[q], maxiter, small_polar_tol(items[q].dtype, tol), infos + q,
                         small_dyn, cap_bytes, sh);
}

__device__ void small_qr_dispatch(const mak_batch_item& it, int positive, mak_info* info,
                                  unsigned char* dyn, int cap_bytes, SmallScratch& sh) {
  switch (it.dtype) {
    case MAK_F64: small_qr_item<double>(it, positive, info, dyn, cap_bytes, sh); break;
    case MAK_C64: small_qr_item<zcomplex>(it, positive, info, dyn, cap_bytes, sh); break;
    case MAK_F32: small_qr_item<float>(it, positive, info, dyn, cap_bytes, sh); break;
    case MAK_C32: small_qr_item<ccomplex>(it, positive, info, dyn, cap_bytes, sh); break;
    default:
      if (threadIdx.x == 0) info->status = MAK_ERR_UNSUPPORTED;
  }
  __syncthreads();  // the shared block is reused by the next item
}

__global__ void __launch_bounds__(SMALL_THREADS)
small_qr_list_kernel(const __grid_constant__ SmallList L, int positive, mak_info* infos,
                     int cap_bytes) {
  extern __shared__ __align__(16) unsigned char small_dyn[];
  __shared__ SmallScratch sh;
  for (int q = blockIdx.x; q < L.count; q += gridDim.x)
    small_qr_dispatch(L.items[q], positive, infos + L.idx[q], small_dyn, cap_bytes, sh);
}

__global__ void __launch_bounds__(SMALL_THREADS)
small_qr_device_kernel(const mak_batch_item* items, int count, int positive, mak_info* infos,
                       int cap_bytes) {
  extern __shared__ __align__(16) unsigned char small_dyn[];
  __shared__ SmallScratch sh;
  for (int q = blockIdx.x; q < count; q += gridDim.x) {
    small_qr_dispatch(items[q], positive, infos + q, small_dyn, cap_bytes, sh);
  }
}

// the largest dynamic shared memory of the small-block kernels on this
// device, raised as their limit once per device
static int small_smem_limit() {
  static PerDevice<int> pd;
  return pd.get([] {
    cudaFuncAttributes fa;
    size_t stat = 4096;
    if (cudaFuncGetAttributes(&fa, small_qr_list_kernel) == cudaSuccess) stat = fa.sharedSizeBytes;
    const int cap = max_smem_optin() - (int)stat - 1024;
    cudaFuncSetAttribute(small_qr_list_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
    cudaFuncSetAttribute(small_qr_device_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         cap);
    cudaFuncSetAttribute(small_polar_list_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         cap);
    cudaFuncSetAttribute(small_polar_device_kernel,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
    return cap;
  });
}

// shared memory a CTA gives its block: MAK_SMALL_QR_BYTES / MAK_SMALL_POLAR_BYTES
// (0 = off), within the device's limit
int small_qr_cap() {
  const int want = (int)tuning(TUNE_SMALL_QR_BYTES);
  if (want <= 0) return 0;
  const int lim = small_smem_limit();
  return want < lim ? want : lim;
}
int small_polar_cap() {
  const int want = (int)tuning(TUNE_SMALL_POLAR_BYTES);
  if (want <= 0) return 0;
  const int lim = small_smem_limit();
  return want < lim ? want : lim;
}

bool small_qr_fits(const mak_batch_item& it, int cap) {
  return cap > 0 && it.m >= 0 && it.n >= 0 && small_qr_bytes(it.dtype, it.m, it.n) <= (size_t)cap;
}

bool small_polar_fits(const mak_batch_item& it, int cap) {
  return cap > 0 && it.n >= 0 && it.m >= it.n &&
         small_polar_bytes(it.dtype, it.m, it.n) <= (size_t)cap;
}

int small_polar_launch(cudaStream_t st, const mak_batch_item* items, const int* which, int count,
                       int maxiter, double tol, mak_info* infos, int cap) {
  static thread_local SmallList L;
  for (int q0 = 0; q0 < count; q0 += SMALL_LIST_MAX) {
    const int cnt = (count - q0) < SMALL_LIST_MAX ? (count - q0) : SMALL_LIST_MAX;
    L.count = cnt;
    for (int q = 0; q < cnt; q++) {
      L.items[q] = items[which[q0 + q]];
      L.idx[q] = which[q0 + q];
    }
    const int grid = cnt < num_sms() ? cnt : num_sms();
    note_launch();
    small_polar_list_kernel<<<grid, SMALL_THREADS, cap, st>>>(L, maxiter, tol, infos, cap);
    MAK_CUDA_TRY(cudaGetLastError());
  }
  return 0;
}

// one persistent launch (per SMALL_LIST_MAX items) over the listed items
int small_qr_launch(cudaStream_t st, const mak_batch_item* items, const int* which, int count,
                    int positive, mak_info* infos, int cap) {
  static thread_local SmallList L;
  for (int q0 = 0; q0 < count; q0 += SMALL_LIST_MAX) {
    const int cnt = (count - q0) < SMALL_LIST_MAX ? (count - q0) : SMALL_LIST_MAX;
    L.count = cnt;
    for (int q = 0; q < cnt; q++) {
      L.items[q] = items[which[q0 + q]];
      L.idx[q] = which[q0 + q];
    }
    const int grid = cnt < num_sms() ? cnt : num_sms();
    note_launch();
    small_qr_list_kernel<<<grid, SMALL_THREADS, cap, st>>>(L, positive, infos, cap);
    MAK_CUDA_TRY(cudaGetLastError());
  }
  return 0;
}

}  // namespace mak

using namespace mak;

extern "C" int mak_batched_qr_compact_device(const mak_batch_item* items, int nitems,
                                             const mak_qr_opts* opts, mak_info* infos,
                                             mak_stream_t stream) {
  if (nitems < 0) return -2;
  if (nitems > 0 && items == nullptr) return -1;
  if (opts == nullptr) return -3;
  if (nitems > 0 && infos == nullptr) return -4;
  if (nitems == 0) return 0;
  const int cap = small_qr_cap();
  if (cap <= 0) return MAK_ERR_UNSUPPORTED;
  const int grid = nitems < num_sms() ? nitems : num_sms();
  note_launch();
  small_qr_device_kernel<<<grid, SMALL_THREADS, cap, (cudaStream_t)stream>>>(
      items, nitems, opts->positive, infos, cap);
  return cudaGetLastError() == cudaSuccess ? 0 : MAK_ERR_CUDA;
}

extern "C" int mak_batched_left_polar_device(const mak_batch_item* items, int nitems,
                                             const mak_polar_opts* opts, mak_info* infos,
                                             mak_stream_t stream) {
  if (nitems < 0) return -2;
  if (nitems > 0 && items == nullptr) return -1;
  if (opts == nullptr) return -3;
  if (nitems > 0 && infos == nullptr) return -4;
  if (opts->maxiter < 1) return -3;
  if (nitems == 0) return 0;
  const int cap = small_polar_cap();
  if (cap <= 0) return MAK_ERR_UNSUPPORTED;
  const int grid = nitems < num_sms() ? nitems : num_sms();
  note_launch();
  small_polar_device_kernel<<<grid, SMALL_THREADS, cap, (cudaStream_t)stream>>>(
      items, nitems, opts->maxiter, opts->tol, infos, cap);
  return cudaGetLastError() == cudaSuccess ? 0 : MAK_ERR_CUDA;
}

extern "C" int mak_small_qr_max_bytes(void) { return small_qr_cap(); }
extern "C" int mak_small_polar_max_bytes(void) { return small_polar_cap(); }
