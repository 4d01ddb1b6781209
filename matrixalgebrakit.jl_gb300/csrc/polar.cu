// Left polar decomposition by the scaled Newton iteration, GB300 native.
//
// Replaces the reference's left_polar!(A, (W, P), ::PolarNewton)
// (src/implementations/polar.jl:99-111) and left_polar_newton!
// (polar.jl:128-166) with _avgdiff! (polar.jl:209-220; GPU kernel
// ext/MatrixAlgebraKitCUDAExt/MatrixAlgebraKitCUDAExt.jl:154-173) and
// project_hermitian! (src/implementations/projections.jl:61-108).
//
//   m > n : A = Q R (qr_run), iterate on X0 = R;   m == n : iterate on X0 = A
//   X <- (g X + X^{-H}/g)/2,   g = sqrt(||X^{-H}||_F / ||X||_F)
//   stop when max|X^{-H}/g - g X| <= tol  or after maxiter iterations
//   W = Q X  (m > n)  or  W = X,     P = herm(W^H A)
//
// The inverse is an in-place blocked Gauss-Jordan elimination with partial
// pivoting (gje_inverse): per block column of 32 a panel kernel (pivot
// search + row exchange + elimination, one barrier per column, panel rows
// resident in shared memory; a thread-block cluster of up to 8 CTAs for
// n <= 2048, a cooperative grid with a bounded global barrier beyond), a
// row-exchange/save kernel
// for the other columns and one rank-32 GEMM update -- 2n^3 flops in total,
// the same count as the reference's LU + inverse.  The Newton update reads
// X^{-H} straight out of the eliminated matrix through the inverse column
// permutation (no separate transpose or permutation pass) and fuses the
// avgdiff step, the scaling and the max-abs convergence measure.  For
// m > n, P is formed as herm(X^H R) (= herm(W^H A) since A = QR, W = QX),
// an n^3 instead of an m n^2 product.
#include "gemm.cuh"
#include "internal.h"
#include "util.cuh"

#include <climits>
#include <mutex>

namespace mak {

constexpr int GJ_NB = 32;
constexpr int GJ_OUTER_NB = 128;  // block column of the mixed-precision path
constexpr int GJ_THREADS = 256;
constexpr int GJ_CLUSTER_ROWS = 256;  // rows per CTA up to which a panel runs as one cluster

template <class T>
struct GjArgs {
  T* X;
  int64_t ldx;
  int n, k0, b, rpc;
  int* piv;
  real_t<T>* part_val;
  int* part_idx;
  T* swapbuf;  // [2][GJ_NB]: row jj by column parity
  T* cand;     // [2][gstride][GJ_NB]: each CTA's pivot candidate row, by column parity
  int gstride;  // allocation stride of the per-CTA partials
  unsigned* bar;
  int* status;
  int* singular;
  const int* skip;  // device stop flag of a fixed-iteration loop (or nullptr)
};

__device__ __forceinline__ double cabs1_(double x) { return fabs(x); }
__device__ __forceinline__ float cabs1_(float x) { return fabsf(x); }
template <class R> __device__ __forceinline__ R cabs1_(cplx<R> x) { return fabs(x.re) + fabs(x.im); }

// (value desc, index asc) arg-max merge
template <class R>
__device__ __forceinline__ void amax_merge(R& v, int& i, R v2, int i2) {
  if (v2 > v || (v2 == v && i2 < i)) { v = v2; i = i2; }
}

template <class T, int SYNC>
__global__ void __launch_bounds__(GJ_THREADS) gje_panel_kernel(GjArgs<T> a) {
  using R = real_t<T>;
  if (skipped(a.skip)) return;  // the same in every CTA: no barrier is reached
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* Ps = reinterpret_cast<T*>(smem_raw);  // rpc x b, ld = rpc
  T* fsh = Ps + (size_t)a.rpc * a.b;        // rpc multipliers of the current column
  __shared__ R sv[32];
  __shared__ int si[32];
  __shared__ T prow[GJ_NB];
  __shared__ T srow[GJ_NB];
  __shared__ T dinv_s;
  __shared__ int pivs, pivq;
  // cluster variant: this CTA's published pivot candidate, candidate row and
  // (its holder) row jj, by column parity, read by the other CTAs through
  // distributed shared memory after the cluster barrier
  __shared__ R x_val[2];
  __shared__ int x_idx[2];
  __shared__ T x_cand[2][GJ_NB];
  __shared__ T x_rowjj[2][GJ_NB];
  constexpr bool kCl = SYNC == SYNC_CLUSTER;
  const int G = gridDim.x, cb = blockIdx.x, tid = threadIdx.x;
  const int lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  const int rpc = a.rpc, b = a.b, k0 = a.k0;
  const int r0 = cb * rpc;
  const int nr = max(0, min(a.n, r0 + rpc) - r0);
  T* Xp = a.X + (int64_t)k0 * a.ldx;
  for (int c = 0; c < b; c++)
    for (int r = tid; r < nr; r += blockDim.x) Ps[r + c * rpc] = Xp[(r0 + r) + (int64_t)c * a.ldx];
  __syncthreads();

  // Per column one grid-wide round: every CTA publishes its local arg-max
  // (value desc, index asc) together with that candidate row, and the CTA
  // holding row jj publishes row jj.  After the barrier every CTA merges the
  // partials in the same fixed order, reads the winning candidate as the
  // pivot row, and the CTA holding the pivot's old row receives row jj: no
  // second round for the exchange.  The published values are
  // double-buffered by column parity (a CTA writes column j+1's slot only
  // after every CTA passed barrier j, i.e. finished reading column j-1's).
  for (int j = 0; j < b; j++) {
    const int jj = k0 + j;
    const int par = j & 1;
    R* pval = a.part_val + par * a.gstride;
    int* pidx = a.part_idx + par * a.gstride;
    T* rowjj = a.swapbuf + par * GJ_NB;
    T* cand = a.cand + (int64_t)par * a.gstride * GJ_NB;
    // ---- local pivot candidate over global rows >= jj
    R best = R(-1);
    int bidx = INT_MAX;
    for (int r = tid; r < nr; r += blockDim.x) {
      const int gr = r0 + r;
      if (gr >= jj) amax_merge(best, bidx, cabs1_(Ps[r + j * rpc]), gr);
    }
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) {
      R v2 = __shfl_xor_sync(0xffffffffu, best, m);
      int i2 = __shfl_xor_sync(0xffffffffu, bidx, m);
      amax_merge(best, bidx, v2, i2);
    }
    if (lane == 0) { sv[wid] = best; si[wid] = bidx; }
    if (jj >= r0 && jj < r0 + nr)
      for (int c = tid; c < b; c += blockDim.x) {
        if constexpr (kCl) x_rowjj[par][c] = Ps[(jj - r0) + c * rpc];
        else rowjj[c] = Ps[(jj - r0) + c * rpc];
      }
    __syncthreads();
    if (wid == 0) {
      R v = lane < nw ? sv[lane] : R(-1);
      int ix = lane < nw ? si[lane] : INT_MAX;
#pragma unroll
      for (int m = 16; m > 0; m >>= 1) {
        R v2 = __shfl_xor_sync(0xffffffffu, v, m);
        int i2 = __shfl_xor_sync(0xffffffffu, ix, m);
        amax_merge(v, ix, v2, i2);
      }
      if (lane == 0) {
        if constexpr (kCl) {
          x_val[par] = v;
          x_idx[par] = ix;
        } else {
          pval[cb] = v;
          pidx[cb] = ix;
        }
        pivs = ix;
      }
    }
    __syncthreads();
    {
      const int li = pivs;  // this CTA's candidate row (global index)
      if (li != INT_MAX)
        for (int c = tid; c < b; c += blockDim.x) {
          if constexpr (kCl) x_cand[par][c] = Ps[(li - r0) + c * rpc];
          else cand[(int64_t)cb * GJ_NB + c] = Ps[(li - r0) + c * rpc];
        }
    }
    if (!panel_sync<SYNC>(a.bar, G, a.status)) return;

    // ---- global pivot (identical in every CTA), then the exchange
    if (wid == 0) {
      R v = R(-1);
      int ix = INT_MAX, iq = -1;
      for (int q = lane; q < G; q += 32) {
        R v2;
        int i2;
        if constexpr (kCl) {
          v2 = dsmem_ld(&x_val[par], (unsigned)q);
          i2 = dsmem_ld(&x_idx[par], (unsigned)q);
        } else {
          v2 = ld_cg(&pval[q]);
          i2 = ld_cg(&pidx[q]);
        }
        if (v2 > v || (v2 == v && i2 < ix)) { v = v2; ix = i2; iq = q; }
      }
#pragma unroll
      for (int m = 16; m > 0; m >>= 1) {
        R v2 = __shfl_xor_sync(0xffffffffu, v, m);
        int i2 = __shfl_xor_sync(0xffffffffu, ix, m);
        int q2 = __shfl_xor_sync(0xffffffffu, iq, m);
        if (v2 > v || (v2 == v && i2 < ix)) { v = v2; ix = i2; iq = q2; }
      }
      if (lane == 0) {
        pivs = (ix == INT_MAX) ? jj : ix;
        pivq = (ix == INT_MAX || ix == jj) ? -1 : iq;
      }
    }
    __syncthreads();
    const int p = pivs, q = pivq;
    // pivot row: the winning CTA's candidate (row jj itself when p == jj)
    if constexpr (kCl) {
      const unsigned own = (unsigned)(jj / rpc);  // the CTA holding row jj
      for (int c = tid; c < b; c += blockDim.x)
        prow[c] = q < 0 ? dsmem_ld(&x_rowjj[par][c], own)
                        : dsmem_ld(&x_cand[par][c], (unsigned)q);
      if (p != jj && p >= r0 && p < r0 + nr)
        for (int c = tid; c < b; c += blockDim.x)
          Ps[(p - r0) + c * rpc] = dsmem_ld(&x_rowjj[par][c], own);
    } else {
      for (int c = tid; c < b; c += blockDim.x)
        prow[c] = q < 0 ? ld_cg(&rowjj[c]) : ld_cg(&cand[(int64_t)q * GJ_NB + c]);
      if (p != jj && p >= r0 && p < r0 + nr)
        for (int c = tid; c < b; c += blockDim.x) Ps[(p - r0) + c * rpc] = ld_cg(&rowjj[c]);
    }
    if (cb == 0 && tid == 0) a.piv[jj] = p;
    __syncthreads();
    if (tid == 0) {
      const T d = prow[j];
      if (d == zero_<T>()) atomicExch(a.singular, 1);
      dinv_s = inv_fast(d);  // once per column: a dependent FP64 chain
    }
    __syncthreads();
    const T dinv = dinv_s;
    // the scaled pivot row, formed once (GB300 issues about 1.6 FP64
    // operations per clock per SM, so the elimination keeps one FMA per
    // element); its own column holds the new pivot-column entry 1/d
    for (int c = tid; c < b; c += blockDim.x) srow[c] = (c == j) ? dinv : prow[c] * dinv;
    __syncthreads();
    // the rows' multipliers f_r = X[r, jj] first, then the elimination with
    // each warp on its own columns (lanes over rows), so that all eight
    // warps share the FP64 work even when a CTA owns only a few dozen rows
    for (int r = tid; r < nr; r += blockDim.x) fsh[r] = Ps[r + j * rpc];
    __syncthreads();
    for (int c = wid; c < b; c += nw) {
      const T sc = srow[c];
      T* pc = Ps + c * rpc;
      for (int r = lane; r < nr; r += 32) {
        if (r0 + r == jj) pc[r] = sc;
        else if (c == j) pc[r] = -(fsh[r] * dinv);
        else pc[r] = fma_(-fsh[r], sc, pc[r]);
      }
    }
    __syncthreads();
  }
  // cluster variant: no CTA leaves (releasing its shared memory) while
  // another may still read its last column's partials
  if constexpr (kCl) panel_sync<SYNC>(a.bar, G, a.status);
  for (int c = 0; c < b; c++)
    for (int r = tid; r < nr; r += blockDim.x) Xp[(r0 + r) + (int64_t)c * a.ldx] = Ps[r + c * rpc];
}

// For every column outside the panel: apply the panel's row exchanges in
// order, save rows k0..k0+b-1 into buf (b x n) and zero them in X.
// Only columns c in [c_lo, c_hi) are touched.
template <class T>
__global__ void gje_laswp_save_kernel(int n, T* X, int64_t ldx, int k0, int b, const int* piv,
                                      T* buf, int c_lo, int c_hi, const int* skip) {
  if (skipped(skip)) return;
  const int c = c_lo + blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= c_hi || (c >= k0 && c < k0 + b)) return;
  T* col = X + (int64_t)c * ldx;
  for (int t = 0; t < b; t++) {
    const int jj = k0 + t, p = piv[jj];
    if (p != jj && p >= 0 && p < n) {
      T x = col[jj];
      col[jj] = col[p];
      col[p] = x;
    }
  }
  for (int t = 0; t < b; t++) {
    buf[t + (int64_t)c * b] = col[k0 + t];
    col[k0 + t] = zero_<T>();
  }
}

__global__ void iota_kernel(int n, int* v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = i;
}

// iperm = inverse of the composed row permutation
__global__ void gje_perm_kernel(int n, const int* piv, int* iperm, const int* skip) {
  if (skipped(skip)) return;
  extern __shared__ int perm[];
  for (int i = threadIdx.x; i < n; i += blockDim.x) perm[i] = i;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int jj = 0; jj < n; jj++) {
      const int p = piv[jj];
      if (p != jj && p >= 0 && p < n) {
        int t = perm[jj];
        perm[jj] = perm[p];
        perm[p] = t;
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) iperm[perm[i]] = i;
}

// slab capacity of the panel kernel; the kernels' dynamic shared-memory
// limits are raised once per type and device
template <class T>
static size_t gj_slab_cap() {
  static PerDevice<size_t> pd;
  return pd.get([] {
    cudaFuncAttributes fa;
    size_t stat = 16 * 1024;
    if (cudaFuncGetAttributes(&fa, gje_panel_kernel<T, SYNC_GRID>) == cudaSuccess)
      stat = fa.sharedSizeBytes;
    if (cudaFuncGetAttributes(&fa, gje_panel_kernel<T, SYNC_CLUSTER>) == cudaSuccess &&
        fa.sharedSizeBytes > stat)
      stat = fa.sharedSizeBytes;
    const size_t cap = (size_t)max_smem_optin() - stat - 1024;
    cudaFuncSetAttribute(gje_panel_kernel<T, SYNC_GRID>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap);
    cudaFuncSetAttribute(gje_panel_kernel<T, SYNC_CLUSTER>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap);
    cudaFuncSetAttribute(gje_perm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         max_smem_optin() - 1024);
    return cap;
  });
}

template <class T>
int gje_inverse(cudaStream_t st, int64_t n, T* X, int64_t ldx, int* iperm, int precision,
                Arena& ar, mak_info* info) {
  const int sms = num_sms();
  // mixed precision: 128-wide block columns, eliminated with 32-wide panels
  // whose updates stay inside the block; the other columns then receive one
  // rank-128 update through the split-precision tensor-core GEMM
  // the 128-wide blocking from n^2 128 >= 2^25 multiply-adds (complex
  // counted 4x: n >= 512 real, n >= 256 complex; MAK_GJ_SPLIT_MIN overrides
  // it).  Below that the native elimination runs even when mixed precision
  // is asked for (a gate of its own: the general split-product gate does not
  // move it).  Measured on the 300 uneven blocks (mixed polar, CUDA-graph
  // replay, 16 streams): gate 2^29 / 2^25 / 2^23 gave 2.23 / 1.80 / 1.75 s;
  // the launches the lower gates add only cost when they are not replayed
  // from a graph (the same batch issued eagerly: 2.68 / 5.47 / 5.64 s).
  const double gate = tuning(TUNE_GJ_SPLIT_MIN);
  const bool mixed = precision == MAK_PREC_MIXED && sizeof(real_t<T>) == 8 &&
                     (traits<T>::cpx ? 4.0 : 1.0) * (double)n * (double)n * GJ_OUTER_NB >= gate;
  const int NBO = mixed ? GJ_OUTER_NB : GJ_NB;
  int* piv = ar.take<int>(n > 0 ? n : 1);
  // per-CTA pivot partials and candidate rows, double-buffered by column parity
  real_t<T>* part_val = ar.take<real_t<T>>(2 * sms);
  int* part_idx = ar.take<int>(2 * sms);
  T* swapbuf = ar.take<T>(2 * GJ_NB);
  T* cand = ar.take<T>((size_t)2 * sms * GJ_NB);
  T* buf = ar.take<T>((size_t)NBO * (n > 0 ? n : 1));
  T* bufo = mixed ? ar.take<T>((size_t)NBO * (n > 0 ? n : 1)) : nullptr;
  unsigned* bar = ar.take<unsigned>(2);
  char* ozs = nullptr;
  size_t oz_bytes = 0;
  if (mixed) {
    Arena meas(nullptr, 0);
    gemm_prec<T>(st, precision, n, n, NBO, one_<T>(), opnd<T>(nullptr, 1), opnd<T>(nullptr, 1),
                 one_<T>(), nullptr, 1, meas, nullptr);
    oz_bytes = meas.off + 1024;
    ozs = ar.take<char>(oz_bytes);
  }
  if (ar.base == nullptr) return 0;
  if (!ar.ok()) return MAK_ERR_WORKSPACE;
  if (n <= 0) return 0;
  if ((size_t)n * sizeof(int) > (size_t)max_smem_optin() - 1024) return MAK_ERR_UNSUPPORTED;
  MAK_CUDA_TRY(cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), st));
  // pivots start as the identity so that an aborted panel (bounded barrier
  // timeout) still leaves every index in range
  note_launch();
  iota_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>((int)n, piv);
  const size_t cap = gj_slab_cap<T>();
  // one 32-wide panel (cooperative launch, at most max_ctas CTAs: on the
  // look-ahead side stream it leaves the other SMs to the main stream)
  auto panel = [&](int64_t k0, int b, cudaStream_t s, int max_ctas) -> int {
    GjArgs<T> ga{X, ldx, (int)n, (int)k0, b, 0, piv, part_val, part_idx, swapbuf,
                 cand, sms, bar, &info->status, &info->singular, skip_flag()};
    // n <= 8 x 256: one thread-block cluster of at most 8 CTAs (>= 64 rows
    // each); clusters of different streams run side by side
    if (n <= (int64_t)kPanelClusterMax * GJ_CLUSTER_ROWS &&
        (size_t)GJ_CLUSTER_ROWS * (b + 1) * sizeof(T) <= cap) {
      int64_t G = ceil_div(n, 64);
      if (G > kPanelClusterMax) G = kPanelClusterMax;
      const int64_t rpc = ceil_div(n, G);
      G = ceil_div(n, rpc);
      ga.rpc = (int)rpc;
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute attr[1];
      cfg.gridDim = dim3((unsigned)G);
      cfg.blockDim = dim3(GJ_THREADS);
      cfg.dynamicSmemBytes = (size_t)rpc * (b + 1) * sizeof(T);
      cfg.stream = s;
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = (unsigned)G;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      int nclusters = 0;
      if (cudaOccupancyMaxActiveClusters(&nclusters, gje_panel_kernel<T, SYNC_CLUSTER>, &cfg) ==
              cudaSuccess &&
          nclusters >= 1) {
        ProfScope prof(s, PROF_GJ_PANEL, 2.0 * (double)n * b * sizeof(T));
        note_launch();
        MAK_CUDA_TRY(cudaLaunchKernelEx(&cfg, gje_panel_kernel<T, SYNC_CLUSTER>, ga));
        return 0;
      }
      (void)cudaGetLastError();  // fall through to the cooperative grid
    }
    // grid: rows per CTA >= 64, at most one CTA per SM, slab within shared memory
    int64_t G = ceil_div(n, 64);
    if (G > max_ctas) G = max_ctas;
    // the slab holds rpc x (b + 1) values: the panel rows and their multipliers
    int64_t rpc = ceil_div(n, G);
    if ((size_t)rpc * (b + 1) * sizeof(T) > cap) {
      G = ceil_div(n, (int64_t)(cap / ((size_t)(b + 1) * sizeof(T))));
      if (G > sms) return MAK_ERR_UNSUPPORTED;
      rpc = ceil_div(n, G);
    }
    G = ceil_div(n, rpc);
    size_t smem = (size_t)rpc * (b + 1) * sizeof(T);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gje_panel_kernel<T, SYNC_GRID>,
                                                      GJ_THREADS, smem) != cudaSuccess ||
        (int64_t)per_sm * sms < G)
      return MAK_ERR_UNSUPPORTED;
    ga.rpc = (int)rpc;
    void* args[] = {&ga};
    ProfScope prof(s, PROF_GJ_PANEL, 2.0 * (double)n * b * sizeof(T));
    note_launch();
    MAK_CUDA_TRY(cudaLaunchCooperativeKernel((void*)gje_panel_kernel<T, SYNC_GRID>,
                                             dim3((unsigned)G), dim3(GJ_THREADS), args, smem, s));
    return 0;
  };
  // the panels of block column [K0, K0 + KB) with their updates confined to
  // the block's columns (the whole elimination when not mixed: KB = n)
  auto factor_block = [&](int64_t K0, int64_t KB, cudaStream_t s, int max_ctas) -> int {
    const int64_t c_lo = K0, c_hi = K0 + KB;
    for (int64_t k0 = K0; k0 < K0 + KB; k0 += GJ_NB) {
      const int b = (int)((K0 + KB - k0) < GJ_NB ? (K0 + KB - k0) : GJ_NB);
      MAK_TRY(panel(k0, b, s, max_ctas));
      note_launch();
      gje_laswp_save_kernel<T><<<(unsigned)ceil_div(c_hi - c_lo, 128), 128, 0, s>>>(
          (int)n, X, ldx, (int)k0, b, piv, buf, (int)c_lo, (int)c_hi, skip_flag());
      MAK_CUDA_TRY(cudaGetLastError());
      const T* F = X + k0 * ldx;
      if (k0 > c_lo)
        MAK_TRY(gemm<T>(s, n, k0 - c_lo, b, one_<T>(), opnd<T>(F, ldx),
                        opnd<T>(buf + c_lo * b, b), one_<T>(), X + c_lo * ldx, ldx));
      if (k0 + b < c_hi)
        MAK_TRY(gemm<T>(s, n, c_hi - k0 - b, b, one_<T>(), opnd<T>(F, ldx),
                        opnd<T>(buf + (k0 + b) * b, b), one_<T>(), X + (k0 + b) * ldx, ldx));
    }
    return 0;
  };
  // block column [K0, K0 + KB) applied to the columns [c_lo, c_hi) outside
  // it: its row exchanges, then one rank-KB update (split-precision product)
  auto apply_block = [&](int64_t K0, int64_t KB, int64_t c_lo, int64_t c_hi, cudaStream_t s,
                         int max_ctas) -> int {
    if (c_hi <= c_lo) return 0;
    note_launch();
    gje_laswp_save_kernel<T><<<(unsigned)ceil_div(c_hi - c_lo, 128), 128, 0, s>>>(
        (int)n, X, ldx, (int)K0, (int)KB, piv, bufo, (int)c_lo, (int)c_hi, skip_flag());
    MAK_CUDA_TRY(cudaGetLastError());
    const T* Fb = X + K0 * ldx;
    const int64_t l1 = c_hi < K0 ? c_hi : K0;  // left part [c_lo, l1)
    if (l1 > c_lo) {
      Arena oz(ozs, oz_bytes);
      MAK_TRY(gemm_prec<T>(s, precision, n, l1 - c_lo, KB, one_<T>(), opnd<T>(Fb, ldx),
                           opnd<T>(bufo + c_lo * KB, KB), one_<T>(), X + c_lo * ldx, ldx, oz,
                           &info->status, max_ctas));
    }
    const int64_t r0 = c_lo > K0 + KB ? c_lo : K0 + KB;  // right part [r0, c_hi)
    if (c_hi > r0) {
      Arena oz(ozs, oz_bytes);
      MAK_TRY(gemm_prec<T>(s, precision, n, c_hi - r0, KB, one_<T>(), opnd<T>(Fb, ldx),
                           opnd<T>(bufo + r0 * KB, KB), one_<T>(), X + r0 * ldx, ldx, oz,
                           &info->status, max_ctas));
    }
    return 0;
  };

  if (!mixed) {
    MAK_TRY(factor_block(0, n, st, sms));
  } else {
    // Look-ahead: block K is applied first to block K+1's columns; the side
    // stream then factors block K+1 (its panels touch only its own columns,
    // and its row exchanges reach the other columns when block K+1 is
    // applied) while the main stream applies block K to the remaining
    // columns.
    const int64_t nblk = ceil_div(n, (int64_t)NBO);
    LookAhead* la = (nblk > 1 && lookahead_enabled() && n >= 2048) ? lookahead() : nullptr;
    const int la_ctas = lookahead_ctas();
    MAK_TRY(factor_block(0, n < NBO ? n : NBO, st, sms));
    for (int64_t K = 0; K < nblk; K++) {
      const int64_t K0 = K * NBO, KB = (n - K0) < NBO ? (n - K0) : NBO;
      const int64_t nx = K0 + KB;
      const bool has_next = nx < n;
      const int64_t nKB = has_next ? ((n - nx) < NBO ? (n - nx) : NBO) : 0;
      if (has_next && la) {
        MAK_TRY(apply_block(K0, KB, nx, nx + nKB, st, 0));
        MAK_CUDA_TRY(cudaEventRecord(la->ev_ready, st));
        MAK_CUDA_TRY(cudaStreamWaitEvent(la->side, la->ev_ready, 0));
        MAK_TRY(factor_block(nx, nKB, la->side, la_ctas));
        MAK_CUDA_TRY(cudaEventRecord(la->ev_done, la->side));
        MAK_TRY(apply_block(K0, KB, 0, K0, st, sms - la_ctas));
        MAK_TRY(apply_block(K0, KB, nx + nKB, n, st, sms - la_ctas));
        MAK_CUDA_TRY(cudaStreamWaitEvent(st, la->ev_done, 0));
      } else {
        MAK_TRY(apply_block(K0, KB, 0, n, st, 0));
        if (has_next) MAK_TRY(factor_block(nx, nKB, st, sms));
      }
    }
  }
  note_launch();
  gje_perm_kernel<<<1, 1024, (size_t)n * sizeof(int), st>>>((int)n, piv, iperm, skip_flag());
  MAK_CUDA_TRY(cudaGetLastError());
  return 0;
}

// ---- Newton step -----------------------------------------------------------
__device__ __forceinline__ void atomic_max_nonneg(double* addr, double v) {
  atomicMax((unsigned long long*)addr, (unsigned long long)__double_as_longlong(v));
}
__device__ __forceinline__ void atomic_max_nonneg(float* addr, float v) {
  atomicMax((unsigned int*)addr, __float_as_uint(v));
}

// X <- (g X + Y^H/g)/2 with Y^H[i,j] = conj(Xi[j, iperm[i]]) (Xi = eliminated
// inverse), g = (||Xi||_F^2 / ||X||_F^2)^(1/4); *conv = max |Y^H/g - g X|.
template <class T>
__global__ void __launch_bounds__(256) newton_update_kernel(int n, T* X, int64_t ldx,
                                                            const T* Xi, int64_t ldi,
                                                            const int* iperm,
                                                            const real_t<T>* nrm2,
                                                            real_t<T>* conv,
                                                            const int* skip) {
  if (skipped(skip)) return;
  using R = real_t<T>;
  __shared__ T t[32][33];
  __shared__ R sh[32];
  const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + r, j = j0 + tx;
    t[r][tx] = (i < n && j < n) ? Xi[j + (int64_t)iperm[i] * ldi] : zero_<T>();  // t[i'][j'] = Xi[j, iperm[i]]
  }
  __syncthreads();
  const R g = sqrt(sqrt(nrm2[1] / nrm2[0]));
  const R ginv = R(1) / g;
  R dmax = R(0);
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + tx, j = j0 + r;
    if (i < n && j < n) {
      const T y = conj_(t[tx][r]) * ginv;
      const T x = g * X[i + (int64_t)j * ldx];
      X[i + (int64_t)j * ldx] = R(0.5) * (x + y);
      dmax = fmax(dmax, abs_(y - x));
    }
  }
  dmax = block_max(dmax, sh);
  if (threadIdx.x == 0) atomic_max_nonneg(conv, dmax);
}

// Newton-Schulz finish (mixed precision, Float64 types): once a Newton step
// measured n * max|D| <= 1/2 (so ||D||_2 <= ||D||_F <= 1/2 and the new
// iterate's singular values lie in [1, 1.05]), the iteration continues with
// X <- X (3 I - X^H X) / 2, two products on the split tensor-core path
// instead of a latency-bound Gauss-Jordan inverse; it converges
// quadratically there (error e -> 1.5 e^2).  Its measure 2 max|dX| is on the
// Newton step's scale (max|D| = 2 max|dX|) and meets the same tolerance.
constexpr double NS_SWITCH = 0.5;  // n * max|D| at which Newton-Schulz takes over

// Z <- 1.5 I - 0.5 Z  (n x n, ld n)
template <class T>
__global__ void ns_prepare_kernel(int n, T* Z, const int* skip) {
  if (skipped(skip)) return;
  using R = real_t<T>;
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % n, j = e / n;
    const T d = (i == j) ? make_scalar<T>(R(1.5), R(0)) : zero_<T>();
    Z[e] = d - R(0.5) * Z[e];
  }
}

// X <- Xn and *conv = max(*conv, 2 max|Xn - X|)
template <class T>
__global__ void __launch_bounds__(256) ns_update_kernel(int64_t nn, T* X, const T* Xn,
                                                        real_t<T>* conv, const int* skip) {
  if (skipped(skip)) return;
  using R = real_t<T>;
  __shared__ R sh[32];
  R dmax = R(0);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x) {
    const T xn = Xn[e];
    dmax = fmax(dmax, abs_(xn - X[e]));
    X[e] = xn;
  }
  dmax = block_max(dmax, sh);
  if (threadIdx.x == 0) atomic_max_nonneg(conv, R(2) * dmax);
}

// Fixed-iteration mode: after each step, count it and stop the loop on the
// device once its measure is within tol (or is not a number), as the
// reference's host loop does; the Newton-Schulz switch is decided here too.
// w: [0] stopped, [1] steps taken, [2] Newton-Schulz phase, [3] skip flag of
// the Newton step's kernels, [4] skip flag of the Newton-Schulz step's.
template <class R>
__global__ void newton_stop_kernel(const R* conv, R tol, int* w, R* conv_last, int n,
                                   int ns_ok) {
  if (w[0]) return;
  w[1] += 1;
  *conv_last = *conv;
  if (!(*conv > tol)) w[0] = 1;
  else if (ns_ok && !w[2] && (R)n * *conv <= (R)NS_SWITCH) w[2] = 1;
  w[3] = w[0] | w[2];
  w[4] = w[0] | !w[2];
}

template <class T>
__global__ void info_polar_fixed_kernel(mak_info* info, const int* stopw,
                                        const real_t<T>* conv_last, real_t<T> tol) {
  info->iterations = stopw[1];
  info->residual = (double)*conv_last;
  info->converged = (*conv_last <= tol) ? 1 : 0;
}

template <class T>
__global__ void info_polar_kernel(mak_info* info, int it, double conv, int converged) {
  info->iterations = it;
  info->residual = conv;
  info->converged = converged;
}

template <class T>
int polar_newton_run(cudaStream_t st, int64_t m, int64_t n, T* A, int64_t lda, T* W, int64_t ldw,
                     T* P, int64_t ldp, int maxiter, double tol, int precision, Arena& ar,
                     mak_info* info) {
  using R = real_t<T>;
  const bool want_p = P != nullptr;
  T* X = ar.take<T>((size_t)n * n + 1);
  T* Y = ar.take<T>((size_t)n * n + 1);
  int* iperm = ar.take<int>(n + 1);
  R* red = ar.take<R>(RED_CTAS + 8);
  int* stopw = ar.take<int>(5);  // fixed-iteration mode: see newton_stop_kernel
  const bool ns_ok = precision == MAK_PREC_MIXED && sizeof(real_t<T>) == 8;
  T* Yn = ns_ok ? ar.take<T>((size_t)n * n + 1) : nullptr;  // Newton-Schulz product
  // Without host synchronization (the batched driver) both step kinds are
  // launched every iteration and flags let one run.  There the finish is
  // used from n >= 256 (MAK_NS_FIXED_MIN_N / _MAX_N override the range):
  // below, the extra launches cost more than the Gauss-Jordan inverses
  // saved.  Measured on the 300 uneven blocks (mixed, CUDA-graph replay, 16
  // streams, tensor-core Gauss-Jordan updates from 2^25): finish for
  // 256 <= n <= 384 only 1.80 s, for every n >= 256 1.54 s.  The
  // host-checked loop launches just the step it takes and uses the finish
  // at every n.
  const double ns_lo = tuning(TUNE_NS_FIXED_MIN_N), ns_hi = tuning(TUNE_NS_FIXED_MAX_N);
  const bool ns_fixed_ok = ns_ok && n >= ns_lo && n <= ns_hi;
  T* Qw = (m > n) ? ar.take<T>((size_t)m * n) : nullptr;
  T* Rw = (m > n) ? ar.take<T>((size_t)n * n) : nullptr;
  T* A0 = (m == n && want_p) ? ar.take<T>((size_t)n * n) : nullptr;
  // the QR (m > n, once) and Gauss-Jordan (every iteration) workspaces are
  // used one after the other, so they share one tail region
  size_t qr_ws = 0, gj_ws = 0;
  if (m > n) {
    Arena meas(nullptr, 0);
    qr_run<T>(st, m, n, nullptr, lda, nullptr, m, n, nullptr, n, n, 1, 0, precision, meas,
              nullptr);
    qr_ws = meas.off + 256;
  }
  {
    Arena meas(nullptr, 0);
    gje_inverse<T>(st, n, nullptr, n, nullptr, precision, meas, nullptr);
    gj_ws = meas.off + 256;
    for (int64_t mm : {m, n}) {  // W = Q X and P = X^H R products
      Arena m2(nullptr, 0);
      gemm_prec<T>(st, precision, mm, n, n, one_<T>(), opnd<T>(nullptr, 1), opnd<T>(nullptr, 1),
                   zero_<T>(), nullptr, 1, m2, nullptr);
      if (m2.off + 256 > gj_ws) gj_ws = m2.off + 256;
    }
  }
  const size_t tail_bytes = qr_ws > gj_ws ? qr_ws : gj_ws;
  // tol < 0: no host synchronization (graph-capturable); the loop launches
  // maxiter iterations and stops on the device once |tol| is reached
  const bool fixed_iters = tol < 0;
  if (fixed_iters) tol = -tol;
  char* tail = ar.take<char>(tail_bytes);
  if (ar.base == nullptr) return 0;
  if (!ar.ok()) return MAK_ERR_WORKSPACE;
  R* nrm2 = red + RED_CTAS;      // [0] ||X||^2, [1] ||Xi||^2
  R* conv = red + RED_CTAS + 2;  // max |D|
  R* conv_last = red + RED_CTAS + 3;

  if (m > n) {
    Arena sub(tail, tail_bytes);
    MAK_TRY(qr_run<T>(st, m, n, A, lda, Qw, m, n, Rw, n, n, 1, 0, precision, sub, info));
    MAK_TRY(copy_mat<T>(st, n, n, Rw, n, X, n));
  } else {
    if (want_p) MAK_TRY(copy_mat<T>(st, n, n, A, lda, A0, n));
    MAK_TRY(copy_mat<T>(st, n, n, A, lda, X, n));
  }
  int it = 0;
  R hconv = R(0);
  bool converged = (n == 0);
  if (fixed_iters) {
    MAK_CUDA_TRY(cudaMemsetAsync(stopw, 0, 4 * sizeof(int), st));
    MAK_CUDA_TRY(cudaMemsetAsync(stopw + 4, 1, sizeof(int), st));  // non-zero: Newton first
    MAK_CUDA_TRY(cudaMemsetAsync(conv_last, 0, sizeof(R), st));
  }
  const int64_t nn = n * n;
  const unsigned gnn = (unsigned)(ceil_div(nn > 0 ? nn : 1, (int64_t)256) < RED_CTAS
                                      ? ceil_div(nn > 0 ? nn : 1, (int64_t)256)
                                      : RED_CTAS);
  // one Newton step: X <- (g X + X^{-H}/g) / 2, measure max|D| into conv
  auto newton_step = [&]() -> int {
    MAK_TRY(copy_mat<T>(st, n, n, X, n, Y, n));
    {
      Arena sub(tail, tail_bytes);
      MAK_TRY(gje_inverse<T>(st, n, Y, n, iperm, precision, sub, info));
    }
    MAK_TRY(reduce_mat<T>(st, n, n, X, n, 0, red, nrm2));
    MAK_TRY(reduce_mat<T>(st, n, n, Y, n, 0, red, nrm2 + 1));
    dim3 g((unsigned)ceil_div(n, 32), (unsigned)ceil_div(n, 32));
    note_launch();
    newton_update_kernel<T><<<g, 256, 0, st>>>((int)n, X, n, Y, n, iperm, nrm2, conv,
                                               skip_flag());
    return cudaGetLastError() == cudaSuccess ? 0 : MAK_ERR_CUDA;
  };
  // one Newton-Schulz step: X <- X (3 I - X^H X) / 2 (Y holds X^H X, then
  // 1.5 I - 0.5 X^H X), measure 2 max|dX| into conv
  auto ns_step = [&]() -> int {
    {
      Arena oz(tail, tail_bytes);
      MAK_TRY(gemm_prec<T>(st, precision, n, n, n, one_<T>(), opnd<T>(X, n, OP_C), opnd<T>(X, n),
                           zero_<T>(), Y, n, oz, &info->status));
    }
    note_launch();
    ns_prepare_kernel<T><<<gnn, 256, 0, st>>>((int)n, Y, skip_flag());
    MAK_CUDA_TRY(cudaGetLastError());
    {
      Arena oz(tail, tail_bytes);
      MAK_TRY(gemm_prec<T>(st, precision, n, n, n, one_<T>(), opnd<T>(X, n), opnd<T>(Y, n),
                           zero_<T>(), Yn, n, oz, &info->status));
    }
    note_launch();
    ns_update_kernel<T><<<gnn, 256, 0, st>>>(nn, X, Yn, conv, skip_flag());
    return cudaGetLastError() == cudaSuccess ? 0 : MAK_ERR_CUDA;
  };
  bool in_ns = false;  // tolerance mode: the host decides the phase
  for (it = 1; it <= maxiter && n > 0; it++) {
    MAK_CUDA_TRY(cudaMemsetAsync(conv, 0, sizeof(R), st));
    if (fixed_iters) {
      // both step kinds are launched; device flags let exactly one run (and
      // neither once the loop has stopped)
      {
        SkipScope skip_newton(stopw + 3);
        MAK_TRY(newton_step());
      }
      if (ns_fixed_ok) {
        SkipScope skip_ns(stopw + 4);
        MAK_TRY(ns_step());
      }
      note_launch();
      newton_stop_kernel<R><<<1, 1, 0, st>>>(conv, (R)tol, stopw, conv_last, (int)n,
                                             ns_fixed_ok ? 1 : 0);
      MAK_CUDA_TRY(cudaGetLastError());
    } else {
      MAK_TRY(in_ns ? ns_step() : newton_step());
      MAK_CUDA_TRY(cudaMemcpyAsync(&hconv, conv, sizeof(R), cudaMemcpyDeviceToHost, st));
      MAK_CUDA_TRY(cudaStreamSynchronize(st));
      if (!(hconv > (R)tol)) {  // also stops on NaN
        converged = hconv <= (R)tol;
        break;
      }
      if (ns_ok && !in_ns && (R)n * hconv <= (R)NS_SWITCH) in_ns = true;
    }
  }
  if (it > maxiter) it = maxiter;
  note_launch();
  if (fixed_iters)
    info_polar_fixed_kernel<T><<<1, 1, 0, st>>>(info, stopw, conv_last, (R)tol);
  else
    info_polar_kernel<T><<<1, 1, 0, st>>>(info, n > 0 ? it : 0, (double)hconv, converged ? 1 : 0);
  MAK_CUDA_TRY(cudaGetLastError());

  auto G = [&](int64_t M_, int64_t N_, int64_t K_, Operand<T> a, Operand<T> b, T* C_,
               int64_t ldc) -> int {
    Arena oz(tail, tail_bytes);
    return gemm_prec<T>(st, precision, M_, N_, K_, one_<T>(), a, b, zero_<T>(), C_, ldc, oz,
                        &info->status);
  };
  if (m > n) {
    MAK_TRY(G(m, n, n, opnd<T>(Qw, m), opnd<T>(X, n), W, ldw));
    if (want_p) {
      MAK_TRY(G(n, n, n, opnd<T>(X, n, OP_C), opnd<T>(Rw, n, OP_N, MASK_UPPER), P, ldp));
      MAK_TRY(herm_project<T>(st, n, P, ldp));
    }
  } else {
    MAK_TRY(copy_mat<T>(st, n, n, X, n, W, ldw));
    if (want_p) {
      MAK_TRY(G(n, n, n, opnd<T>(X, n, OP_C), opnd<T>(A0, n), P, ldp));
      MAK_TRY(herm_project<T>(st, n, P, ldp));
    }
  }
  return 0;
}

#define MAK_INST_POLAR(T)                                                                     \
  template int gje_inverse<T>(cudaStream_t, int64_t, T*, int64_t, int*, int, Arena&,          \
                              mak_info*);                                                     \
  template int polar_newton_run<T>(cudaStream_t, int64_t, int64_t, T*, int64_t, T*, int64_t, \
                                   T*, int64_t, int, double, int, Arena&, mak_info*);
MAK_INST_POLAR(double)
MAK_INST_POLAR(float)
MAK_INST_POLAR(zcomplex)
MAK_INST_POLAR(ccomplex)

template <class T>
static double default_tol() {
  // defaulttol = eps(real T)^(2/3)  (src/common/defaults.jl:10)
  return pow(sizeof(real_t<T>) == 8 ? 2.220446049250313e-16 : 1.1920928955078125e-7, 2.0 / 3.0);
}

template <class T>
static int polar_entry(int64_t m, int64_t n, void* Av, int64_t lda, void* Wv, int64_t ldw,
                       void* Pv, int64_t ldp, const mak_polar_opts* opts, void* work,
                       size_t work_bytes, mak_info* info, mak_stream_t stream) {
  T* A = (T*)Av;
  T* W = (T*)Wv;
  T* P = (T*)Pv;
  if (m < 0) return -1;
  if (n < 0 || n > m) return -2;  // m >= n required (polar.jl:9-10)
  if (A == nullptr && m * n > 0) return -3;
  if (lda < (m > 1 ? m : 1)) return -4;
  if (W == nullptr && m * n > 0) return -5;
  if ((void*)W == (void*)A && m * n > 0) return -5;
  if (ldw < (m > 1 ? m : 1)) return -6;
  if (P != nullptr && ldp < (n > 1 ? n : 1)) return -8;
  mak_polar_opts o{10, MAK_PREC_NATIVE, 0.0};
  if (opts) o = *opts;
  if (o.maxiter < 1) return -9;
  if (o.precision != MAK_PREC_NATIVE && o.precision != MAK_PREC_MIXED) return -9;
  // tol < 0 selects the fixed-iteration (no host sync) mode, reported
  // against the default tolerance
  const double tol = o.tol > 0 ? o.tol : (o.tol < 0 ? -default_tol<T>() : default_tol<T>());
  if (info == nullptr) return -12;
  cudaStream_t st = (cudaStream_t)stream;
  {
    Arena meas(nullptr, 0);
    polar_newton_run<T>(st, m, n, nullptr, lda, nullptr, ldw, P, ldp, o.maxiter, tol, o.precision,
                        meas, nullptr);
    if (meas.off > work_bytes) return -11;
  }
  Arena ar(work, work_bytes);
  MAK_TRY(info_reset(st, info));
  return polar_newton_run<T>(st, m, n, A, lda, W, ldw, P, ldp, o.maxiter, tol, o.precision, ar,
                             info);
}

}  // namespace mak

using namespace mak;

extern "C" {

int mak_left_polar_workspace(int dtype, int64_t m, int64_t n, int want_p,
                             const mak_polar_opts* opts, size_t* bytes) {
  if (bytes == nullptr) return -6;
  if (m < 0) return -2;
  if (n < 0 || n > m) return -3;
  mak_polar_opts o{10, MAK_PREC_NATIVE, 0.0};
  if (opts) o = *opts;
  Arena meas(nullptr, 0);
  void* P = want_p ? (void*)16 : nullptr;  // only nullness matters when measuring
  switch (dtype) {
    case MAK_F64: polar_newton_run<double>(0, m, n, nullptr, m, nullptr, m, (double*)P, n, o.maxiter, 1.0, o.precision, meas, nullptr); break;
    case MAK_C64: polar_newton_run<zcomplex>(0, m, n, nullptr, m, nullptr, m, (zcomplex*)P, n, o.maxiter, 1.0, o.precision, meas, nullptr); break;
    case MAK_F32: polar_newton_run<float>(0, m, n, nullptr, m, nullptr, m, (float*)P, n, o.maxiter, 1.0, o.precision, meas, nullptr); break;
    case MAK_C32: polar_newton_run<ccomplex>(0, m, n, nullptr, m, nullptr, m, (ccomplex*)P, n, o.maxiter, 1.0, o.precision, meas, nullptr); break;
    default: return -1;
  }
  *bytes = meas.off + 256;
  return 0;
}

#define MAK_POLAR_ENTRY(NAME, T, PT)                                                            \
  int NAME(int64_t m, int64_t n, PT* A, int64_t lda, PT* W, int64_t ldw, PT* P, int64_t ldp,    \
           const mak_polar_opts* opts, void* work, size_t work_bytes, mak_info* info,           \
           mak_stream_t stream) {                                                               \
    return polar_entry<T>(m, n, A, lda, W, ldw, P, ldp, opts, work, work_bytes, info, stream); \
  }
MAK_POLAR_ENTRY(mak_left_polar_newton_d, double, double)
MAK_POLAR_ENTRY(mak_left_polar_newton_z, zcomplex, void)
MAK_POLAR_ENTRY(mak_left_polar_newton_s, float, float)
MAK_POLAR_ENTRY(mak_left_polar_newton_c, ccomplex, void)

}  // extern "C"
