// Internal (C++) interfaces shared between the translation units of
// libmak_gb300.so.  Each template is explicitly instantiated for double,
// zcomplex, float and ccomplex in the .cu file that defines it.
#pragma once
#include <cstdlib>
#include "mak_common.cuh"

namespace mak {

// Blocked Householder QR of A (m x n, destroyed) producing Q (m x qcols,
// qcols = min(m,n) compact or m full) and optionally R (rrows x n).
// Workspace from `ar`; with ar.base == nullptr only sizes are accumulated.
template <class T>
int qr_run(cudaStream_t st, int64_t m, int64_t n, T* A, int64_t lda, T* Q, int64_t ldq,
           int64_t qcols, T* R, int64_t ldr, int64_t rrows, int positive, int blocksize,
           int precision, Arena& ar, mak_info* info);

// In-place inverse of the n x n matrix X (Gauss-Jordan with partial
// pivoting).  On return X holds inv(P X) where P is the row permutation;
// `iperm` (n ints) receives the inverse permutation so that
// inv(X)[:, c] = Xout[:, iperm[c]].
template <class T>
int gje_inverse(cudaStream_t st, int64_t n, T* X, int64_t ldx, int* iperm, int precision,
                Arena& ar, mak_info* info);

int info_reset(cudaStream_t st, mak_info* info);

// qr_pullback! (dA += ...); known_p >= 0 skips the host read of the rank
template <class T>
int qr_pullback_run(cudaStream_t st, int64_t m, int64_t n, int full, T* dA, int64_t ldda,
                    const T* Q, int64_t ldq, const T* R, int64_t ldr, const T* dQ, int64_t lddq,
                    const T* dR, int64_t lddr, double rank_atol, double gauge_atol, int precision,
                    Arena& ar, mak_info* info, int known_p = -1);
// numerical rank of the k x n triangular R into the device int *p_out
template <class T>
int qr_rank_run(cudaStream_t st, int64_t k, int64_t n, const T* R, int64_t ldr, double rank_atol,
                Arena& ar, int* p_out);
// left_polar_pullback! (dA += ...); maxiter < 0: the Sylvester sign
// iteration runs -maxiter steps stopped on the device (no host sync)
template <class T>
int polar_pullback_run(cudaStream_t st, int64_t m, int64_t n, T* dA, int64_t ldda, const T* W,
                       int64_t ldw, const T* P, int64_t ldp, const T* dW, int64_t lddw,
                       const T* dP, int64_t lddp, int maxiter, int precision, Arena& ar,
                       mak_info* info);

// Tuning parameters of the drivers (tuning.cu): the value set through
// mak_tuning_set, else the environment variable of the same name, else the
// built-in default.  Read at every use, so a table loaded by the caller
// takes effect for the calls that follow.
enum TuneId {
  TUNE_BATCH_STREAMS = 0,    // internal streams of the batched calls
  TUNE_BATCH_GEMM_CTAS,      // per-product CTA cap inside a batched call
  TUNE_SIGN_FIXED_ITERS,     // sign-iteration steps of the batched polar pullback
  TUNE_SPLIT_MIN_MNK,        // smallest product (multiply-adds) taking the split path
  TUNE_GJ_SPLIT_MIN,         // n^2 128 from which Gauss-Jordan blocks by 128 (mixed)
  TUNE_NS_FIXED_MIN_N,       // Newton-Schulz finish in the batched polar: n range
  TUNE_NS_FIXED_MAX_N,
  TUNE_QR_OUTER64_MAX_N,     // mixed QR: 64-wide outer blocks up to this n
  TUNE_LOOKAHEAD_CTAS,       // SMs of the look-ahead side stream
  TUNE_PANEL_HIER_C,         // tall panels: cooperative grid of clusters of this size (0: off)
  TUNE_PANEL_PAIR,           // QR panels: two columns per barrier round (1) or one (0)
  TUNE_OZ_MERGED,            // split GEMM: one MMA per A plane over up to 4 B planes (1)
  TUNE_OZ_NARROW,            // split GEMM, K <= 128: 32-wide tiles, two accumulator sets (1)
  TUNE_LOOKAHEAD_TAIL_COLS,  // far columns from which down the side stream gets more SMs
  TUNE_LOOKAHEAD_TAIL_CTAS,  // the side stream's SMs in that tail
  TUNE_SMALL_QR_BYTES,       // batched QR: blocks up to this many bytes take the one-CTA kernel
  TUNE_SMALL_POLAR_BYTES,    // batched polar: the same for the one-CTA polar kernel
  TUNE_QR_PANEL_SPLIT,       // mixed QR: within-block panel updates as split products (1)
  TUNE_COUNT
};
double tuning(int id);

// one-CTA Householder QR of small blocks from a work list (small.cu): the
// shared memory a CTA gives its block (0: off), whether an item fits, and
// one persistent launch over the listed items (`which` indexes `items` and
// `infos`)
int small_qr_cap();
bool small_qr_fits(const mak_batch_item& it, int cap);
int small_qr_launch(cudaStream_t st, const mak_batch_item* items, const int* which, int count,
                    int positive, mak_info* infos, int cap);
// the same for the one-CTA left polar (PolarNewton), blocks with m >= n
int small_polar_cap();
bool small_polar_fits(const mak_batch_item& it, int cap);
int small_polar_launch(cudaStream_t st, const mak_batch_item* items, const int* which, int count,
                       int maxiter, double tol, mak_info* infos, int cap);

// Look-ahead (QR and Gauss-Jordan): a high-priority side stream factors the
// next block while the main stream updates the far columns.  On/off for
// calls made from the current thread; the side stream and its events belong
// to the calling thread (nullptr if they could not be created); the side
// stream's kernels use lookahead_ctas() SMs and the main stream's persistent
// tensor-core grid the rest.
bool lookahead_enabled();
void set_lookahead(bool on);
struct LookAhead {
  cudaStream_t side;
  cudaEvent_t ev_ready, ev_done;
};
LookAhead* lookahead();
int lookahead_ctas();

// Default cap on the persistent split-GEMM grid for calls made from the
// current thread (0: one CTA per SM).  The batched driver lowers it so that
// the products of blocks on different streams run side by side instead of
// one persistent grid holding every SM.
int split_gemm_cta_budget();
void set_split_gemm_cta_budget(int ctas);

// Scoped form of the two thread-local settings above: the previous values
// come back on every exit path of the scope.
struct ThreadSettingsScope {
  bool lookahead_prev;
  int budget_prev;
  ThreadSettingsScope(bool lookahead_on, int gemm_budget)
      : lookahead_prev(lookahead_enabled()), budget_prev(split_gemm_cta_budget()) {
    set_lookahead(lookahead_on);
    set_split_gemm_cta_budget(gemm_budget);
  }
  ~ThreadSettingsScope() {
    set_lookahead(lookahead_prev);
    set_split_gemm_cta_budget(budget_prev);
  }
  ThreadSettingsScope(const ThreadSettingsScope&) = delete;
  ThreadSettingsScope& operator=(const ThreadSettingsScope&) = delete;
};

// Left polar decomposition by scaled Newton (W m x n, P n x n or nullptr);
// tol < 0 selects the fixed-iteration, host-sync-free mode.
template <class T>
int polar_newton_run(cudaStream_t st, int64_t m, int64_t n, T* A, int64_t lda, T* W, int64_t ldw,
                     T* P, int64_t ldp, int maxiter, double tol, int precision, Arena& ar,
                     mak_info* info);

}  // namespace mak

#include "gemm.cuh"

namespace mak {

// Split-precision (Ozaki scheme, bf16 tcgen05) GEMM for Float64 / ComplexF64:
// C = alpha op(A) op(B) + beta C with real alpha, beta.  Workspace from `ar`
// (measured when ar.base == nullptr).
// max_ctas > 0 caps the persistent grid (so that a kernel on another stream
// keeps SMs of its own); 0 = one CTA per SM.
template <class T>
int oz_gemm(cudaStream_t st, int64_t M, int64_t N, int64_t K, T alpha, Operand<T> A, Operand<T> B,
            T beta, T* C, int64_t ldc, Arena& ar, int* status, int max_ctas = 0);

// Internal precision code: the split product at every size (used by the
// C-ABI GEMM, whose caller chose the arithmetic explicitly).
constexpr int PREC_SPLIT_ALWAYS = 3;
// Inside the factorizations, MAK_PREC_MIXED splits products with at least
// split_min_mnk() multiply-adds (complex counted 4x; 2^22 by default,
// MAK_SPLIT_MIN_MNK overrides it, read once); smaller ones stay native.  The
// QR's mixed blocking is gated by the same value (Gauss-Jordan's has its own).
double split_min_mnk();

// Dispatch: the tensor-core split GEMM when `precision` is MAK_PREC_MIXED and
// the element type is a Float64 type with real alpha/beta, else the native
// SIMT GEMM.  `ar` supplies the split planes (sized by a measuring pass).
template <class T>
int gemm_prec(cudaStream_t st, int precision, int64_t M, int64_t N, int64_t K, T alpha,
              Operand<T> A, Operand<T> B, T beta, T* C, int64_t ldc, Arena& ar, int* status,
              int max_ctas = 0);

}  // namespace mak
