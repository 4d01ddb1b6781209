/*
 * mak_gb300.h -- C ABI of the GB300 (sm_103a) orthogonal-factorization library
 * (libmak_gb300.so), the drop-in for MatrixAlgebraKit.jl's dense QR / polar
 * hot path on CuArrays.
 *
 * Conventions (shared by every entry point):
 *  - column-major storage, 0-based, explicit leading dimensions (ld >= rows);
 *  - element-type suffix: _d Float64, _z ComplexF64, _s Float32, _c ComplexF32;
 *    complex values are interleaved (re, im), i.e. Julia's ComplexF64 layout;
 *  - all matrix pointers are DEVICE pointers owned by the caller; the library
 *    never allocates or frees device memory itself: scratch comes from the
 *    caller's `work` buffer, sized by the matching *_workspace query (the
 *    LAPACK lwork = -1 pattern, reference src/yalapack.jl:179-196);
 *  - calls are stream ordered on `stream` (a cudaStream_t / CUstream; NULL is
 *    the legacy default stream) and do not synchronize the host unless stated;
 *  - return value: 0 ok; -i argument i is invalid (LAPACK convention);
 *    >= 1000 a CUDA launch error (MAK_ERR_*).  Numerical outcomes are written
 *    to the caller's DEVICE `mak_info` record, read whenever the caller
 *    chooses (no hidden synchronization).
 */
#ifndef MAK_GB300_H
#define MAK_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef void* mak_stream_t; /* cudaStream_t */

/* element type codes (used by the workspace queries) */
enum { MAK_F64 = 0, MAK_C64 = 1, MAK_F32 = 2, MAK_C32 = 3 };

/* arithmetic used for the large products */
enum {
  MAK_PREC_NATIVE = 0, /* every flop in the element type's own precision       */
  MAK_PREC_MIXED = 1   /* large GEMMs as split-precision bf16 tensor-core
                          products with exact fp32 accumulation (Ozaki scheme);
                          panels, tau, signs and reductions stay native        */
};

/* host return codes and device status values */
enum {
  MAK_OK = 0,
  MAK_ERR_CUDA = 1000,        /* a kernel launch / runtime call failed       */
  MAK_ERR_TIMEOUT = 1001,     /* a bounded device-side wait gave up          */
  MAK_ERR_UNSUPPORTED = 1002, /* shape outside the supported envelope        */
  MAK_ERR_WORKSPACE = 1003    /* `work_bytes` smaller than the query result  */
};

/* Device-side outcome record (the caller passes a device pointer). */
typedef struct {
  int32_t status;     /* 0 ok, else MAK_ERR_* raised on the device            */
  int32_t iterations; /* Newton / sign-function iterations performed          */
  int32_t rank;       /* numerical rank p used by the QR pullback             */
  int32_t converged;  /* 1 when the Newton stopping test was met              */
  double residual;    /* last Newton residual  max|X^-H/g - g X|              */
  double gauge;       /* pullback: size of the gauge-dependent cotangent part */
  double gauge_atol;  /* pullback: the tolerance it was compared against      */
  int32_t singular;   /* 1 when an exact zero pivot was met in an inverse     */
  int32_t pad;
} mak_info;

/* Options of Householder(; positive, blocksize) (reference
 * src/interface/decompositions.jl:80-86).  pivoted=true is not provided. */
typedef struct {
  int32_t positive;  /* 1 (reference default): diag(R) made real >= 0        */
  int32_t blocksize; /* 0: library default panel width (32); else 1..32;
                        larger values are rejected (-9)                     */
  int32_t precision; /* MAK_PREC_NATIVE or MAK_PREC_MIXED                     */
  int32_t reserved;
} mak_qr_opts;

/* Options of PolarNewton(; maxiter, tol) (reference
 * src/implementations/polar.jl:128). */
typedef struct {
  int32_t maxiter;   /* reference default 10                                  */
  int32_t precision; /* MAK_PREC_NATIVE or MAK_PREC_MIXED                     */
  double tol;        /* > 0: stopping tolerance; 0: reference default
                        eps(real T)^(2/3); < 0: no host synchronization
                        (CUDA-graph capturable): maxiter iterations are
                        launched and the loop stops on the device once the
                        default tolerance is met; the stopped iterations'
                        kernels return at once                              */
} mak_polar_opts;

/* Options of the pullbacks (reference src/pullbacks/qr.jl:73-77). */
typedef struct {
  double rank_atol;  /* < 0: reference default eps(norm(R, Inf))^(3/4)        */
  double gauge_atol; /* < 0: reference default eps(norm(dQ, Inf))^(3/4)       */
  int32_t precision;
  int32_t reserved;
} mak_pullback_opts;

/* library identification */
const char* mak_version(void);
const char* mak_status_string(int code);
/* number of CUDA kernels this library has launched in the process so far
 * (profiling aid: a benchmark reads it before and after its timed region) */
uint64_t mak_kernel_launches(void);

/* Optional device-time accounting per kernel class: between start and stop,
 * launches of the instrumented classes are bracketed by CUDA events on their
 * stream; read waits for those events and returns the summed elapsed time,
 * the summed algorithmic work (flops or bytes) and the launch count.
 * kind: 0 native GEMM, 1 mixed-precision GEMM, 2 QR panel, 3 Gauss-Jordan
 * panel, -1 all. */
int mak_profile_start(void);
int mak_profile_stop(void);
int mak_profile_read(int kind, double* total_ms, double* total_work, uint64_t* launches);

/* Tuning parameters of the drivers (no counterpart in the reference, whose
 * drivers are LAPACK's / CUSOLVER's own): thresholds and counts that choose
 * between code paths and launch shapes.  A parameter's value is the one set
 * here, else the environment variable of the same name, else the built-in
 * default (measured best on a GB300); it is read at every use, process wide,
 * so set a table before the calls it should affect.  Names:
 *   MAK_BATCH_STREAMS      internal streams of the batched calls (1..32, 32)
 *   MAK_BATCH_GEMM_CTAS    CTA cap of each split product in a batched call
 *                          (8..1024, a quarter of the SMs)
 *   MAK_SIGN_FIXED_ITERS   Sylvester sign steps of the batched polar pullback
 *                          (4..200, 30)
 *   MAK_SPLIT_MIN_MNK      smallest product (multiply-adds, complex 4x) that
 *                          takes the split tensor-core path (2^22)
 *   MAK_GJ_SPLIT_MIN       n^2 128 (complex 4x) from which the mixed
 *                          Gauss-Jordan inverse blocks by 128 (2^25)
 *   MAK_NS_FIXED_MIN_N / MAK_NS_FIXED_MAX_N  n range of the Newton-Schulz
 *                          finish in the batched polar (256 .. 2^30)
 *   MAK_QR_OUTER64_MAX_N   mixed QR: 64-wide outer blocks up to this n (0)
 *   MAK_LOOKAHEAD_CTAS     SMs of the look-ahead side stream (8..120, 48)
 *   MAK_PANEL_HIER_C       QR panels too tall for one cluster: 0 = one grid
 *                          barrier over all panel CTAs; 2, 4 or 8 = clusters
 *                          of that many CTAs combine through distributed
 *                          shared memory and only their leaders meet at the
 *                          grid barrier (0)
 *   MAK_PANEL_PAIR         QR panels: two columns per barrier round where the
 *                          norms allow (1), or one (0)
 *   MAK_OZ_MERGED          split GEMM: one MMA per A plane over up to four B
 *                          planes (1), or one MMA per plane pair (0)
 *   MAK_OZ_NARROW          split GEMM with K <= 128: 32-wide tiles with two
 *                          accumulator sets (1), or 64-wide tiles (0)
 *   MAK_LOOKAHEAD_TAIL_COLS / MAK_LOOKAHEAD_TAIL_CTAS  from this many far
 *                          columns down, the look-ahead side stream takes
 *                          this many SMs (4096, 96)
 *   MAK_SMALL_QR_BYTES     batched QR: blocks of at most this many bytes (m n
 *                          + 2 min(m,n) elements) are factored by the one-CTA
 *                          small-block kernel (0 = off; 200704)
 *   MAK_SMALL_POLAR_BYTES  batched polar: the same for the one-CTA Newton
 *                          iteration (0 = off; 200704)
 *   MAK_QR_PANEL_SPLIT     mixed QR: a 32-wide panel's update of the rest of
 *                          its 128-wide block as split tensor-core products
 *                          (1), or on the FP64 pipe (0)
 * mak_tuning_set: 0 ok, -1 unknown name, -2 value out of range; a NaN value
 * returns the parameter to its environment / default value.
 * mak_tuning_get: the value in effect.  mak_tuning_name(i): the i-th name,
 * NULL past the last. */
int mak_tuning_set(const char* name, double value);
int mak_tuning_get(const char* name, double* value);
const char* mak_tuning_name(int index);

/* Self-test of the failure path of the bounded device-side waits (no
 * counterpart in the reference, whose waits are inside LAPACK / CUSOLVER).
 * Launches `ctas` co-resident CTAs that meet at the grid barrier the panel
 * kernels use, expecting ctas + `missing` arrivals, each CTA polling at most
 * `spin_limit` times (1 .. 2^22).  With missing > 0 the wait gives up and
 * the DEVICE int *status becomes MAK_ERR_TIMEOUT; with missing = 0 it stays
 * 0.  `work` is a device buffer of at least 8 bytes.  The kernel always
 * returns and the context stays usable. */
int mak_selftest_barrier(int ctas, int missing, int64_t spin_limit, void* work,
                         size_t work_bytes, int* status, mak_stream_t stream);

/* ------------------------------------------------------------------- QR ---
 * qr_compact!(A, (Q, R), GB300_HouseholderQR(; positive, blocksize))
 * Replaces the reference's qr_householder! (src/implementations/qr.jl:132-188:
 * geqrt!/geqrf! + gemqrt!/unmqr! + uppertriangular! copy + gaugefix!).
 * A (m x n) is destroyed (it holds the packed reflectors on return).
 * Q: m x min(m,n).  R: min(m,n) x n, or NULL (reference: empty R = not wanted,
 * qr.jl:149).  qr_full: Q m x m, R m x n (qr.jl:106-109).
 */
int mak_qr_workspace(int dtype, int64_t m, int64_t n, int full,
                     const mak_qr_opts* opts, size_t* bytes);
int mak_qr_compact_d(int64_t m, int64_t n, double* A, int64_t lda, double* Q, int64_t ldq,
                     double* R, int64_t ldr, const mak_qr_opts* opts, void* work,
                     size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_qr_compact_z(int64_t m, int64_t n, void* A, int64_t lda, void* Q, int64_t ldq,
                     void* R, int64_t ldr, const mak_qr_opts* opts, void* work,
                     size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_qr_compact_s(int64_t m, int64_t n, float* A, int64_t lda, float* Q, int64_t ldq,
                     float* R, int64_t ldr, const mak_qr_opts* opts, void* work,
                     size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_qr_compact_c(int64_t m, int64_t n, void* A, int64_t lda, void* Q, int64_t ldq,
                     void* R, int64_t ldr, const mak_qr_opts* opts, void* work,
                     size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_qr_full_d(int64_t m, int64_t n, double* A, int64_t lda, double* Q, int64_t ldq,
                  double* R, int64_t ldr, const mak_qr_opts* opts, void* work,
                  size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_qr_full_z(int64_t m, int64_t n, void* A, int64_t lda, void* Q, int64_t ldq,
                  void* R, int64_t ldr, const mak_qr_opts* opts, void* work,
                  size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_qr_full_s(int64_t m, int64_t n, float* A, int64_t lda, float* Q, int64_t ldq,
                  float* R, int64_t ldr, const mak_qr_opts* opts, void* work,
                  size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_qr_full_c(int64_t m, int64_t n, void* A, int64_t lda, void* Q, int64_t ldq,
                  void* R, int64_t ldr, const mak_qr_opts* opts, void* work,
                  size_t work_bytes, mak_info* info, mak_stream_t stream);

/* -------------------------------------------------------------------- LQ ---
 * lq_compact!(A, (L, Q), LQViaTransposedQR(GB300_HouseholderQR(; positive)))
 * Replaces the reference's lq_compact! / lq_full! (src/implementations/lq.jl)
 * through its transposed-QR algorithm (LQViaTransposedQR,
 * src/interface/decompositions.jl:340-353): A = L Q is computed as the
 * conjugate transpose of the QR of A^H.  A (m x n) is read, not destroyed.
 * lq_compact: L m x min(m,n) (or NULL: not wanted), Q min(m,n) x n;
 * lq_full: L m x n (or NULL), Q n x n.  positive = 1 gives diag(L) real >= 0.
 */
int mak_lq_workspace(int dtype, int64_t m, int64_t n, int full, const mak_qr_opts* opts,
                     size_t* bytes);
int mak_lq_compact_d(int64_t m, int64_t n, const double* A, int64_t lda, double* L, int64_t ldl,
                     double* Q, int64_t ldq, const mak_qr_opts* opts, void* work,
                     size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_lq_compact_z(int64_t m, int64_t n, const void* A, int64_t lda, void* L, int64_t ldl,
                     void* Q, int64_t ldq, const mak_qr_opts* opts, void* work,
                     size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_lq_compact_s(int64_t m, int64_t n, const float* A, int64_t lda, float* L, int64_t ldl,
                     float* Q, int64_t ldq, const mak_qr_opts* opts, void* work,
                     size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_lq_compact_c(int64_t m, int64_t n, const void* A, int64_t lda, void* L, int64_t ldl,
                     void* Q, int64_t ldq, const mak_qr_opts* opts, void* work,
                     size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_lq_full_d(int64_t m, int64_t n, const double* A, int64_t lda, double* L, int64_t ldl,
                  double* Q, int64_t ldq, const mak_qr_opts* opts, void* work, size_t work_bytes,
                  mak_info* info, mak_stream_t stream);
int mak_lq_full_z(int64_t m, int64_t n, const void* A, int64_t lda, void* L, int64_t ldl,
                  void* Q, int64_t ldq, const mak_qr_opts* opts, void* work, size_t work_bytes,
                  mak_info* info, mak_stream_t stream);
int mak_lq_full_s(int64_t m, int64_t n, const float* A, int64_t lda, float* L, int64_t ldl,
                  float* Q, int64_t ldq, const mak_qr_opts* opts, void* work, size_t work_bytes,
                  mak_info* info, mak_stream_t stream);
int mak_lq_full_c(int64_t m, int64_t n, const void* A, int64_t lda, void* L, int64_t ldl,
                  void* Q, int64_t ldq, const mak_qr_opts* opts, void* work, size_t work_bytes,
                  mak_info* info, mak_stream_t stream);

/* qr_compact! in Float64 that allocates nothing at call time.  It has no
 * counterpart in the reference (whose CUDA path lets CUSOLVER allocate its
 * own workspace).  For callers that cannot allocate device memory or keep a
 * workspace: a caller whose device memory all belongs to its own pool
 * allocator, or a binding with nowhere to keep a buffer between calls.
 * Same arguments, results and errors as mak_qr_compact_d without the
 * workspace; its scratch is one fixed device array of
 * MAK_QR_NOALLOC_SCRATCH_BYTES inside the library.
 *  - With MAK_PREC_MIXED, a problem whose split products' planes do not fit
 *    the array runs the native blocking instead (both are FP64-accurate).
 *    A problem whose native mak_qr_workspace size exceeds the array is
 *    rejected with MAK_ERR_WORKSPACE before any work is queued.
 *  - The first call on each device (made with that device current) looks up
 *    the array's address; it must come before any stream capture starts on
 *    that device.
 *  - Nothing in the array has to start at zero.
 *  - All calls on one device share the array: calls whose executions overlap
 *    (unordered streams, or several host threads) race on it.  Order them on
 *    one stream or with events.
 *  - info must be a device pointer (not NULL). */
#define MAK_QR_NOALLOC_SCRATCH_BYTES ((size_t)32 << 20)
int mak_qr_compact_d_noalloc(int64_t m, int64_t n, double* A, int64_t lda, double* Q,
                             int64_t ldq, double* R, int64_t ldr, const mak_qr_opts* opts,
                             mak_info* info, mak_stream_t stream);

/* ----------------------------------------------------------------- GEMM ---
 * C = alpha op(A) op(B) + beta C, op in {0: N, 1: T, 2: C (conjugate
 * transpose)}.  The product kernel every factorization above uses, exposed
 * so callers can run their own contractions with the same precision control
 * (reference: the mul! calls of src/implementations/polar.jl:63,108,163 and
 * src/pullbacks/{qr,polar}.jl, which go to cuBLAS through CUDA.jl).
 * precision = MAK_PREC_MIXED: Float64 data is split into eight balanced 7-bit
 * bf16 digit planes and the 36 plane pairs of significant weight are
 * multiplied on the tcgen05 tensor cores with exact fp32 group accumulation
 * (Ozaki scheme); alpha/beta must then be real.
 */
int mak_gemm_workspace(int dtype, int opA, int opB, int64_t m, int64_t n, int64_t k,
                       int precision, size_t* bytes);
int mak_gemm_d(int opA, int opB, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
               int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
               int precision, void* work, size_t work_bytes, mak_info* info,
               mak_stream_t stream);
int mak_gemm_z(int opA, int opB, int64_t m, int64_t n, int64_t k, const double* alpha,
               const void* A, int64_t lda, const void* B, int64_t ldb, const double* beta,
               void* C, int64_t ldc, int precision, void* work, size_t work_bytes,
               mak_info* info, mak_stream_t stream);

/* ---------------------------------------------------------------- polar ---
 * left_polar!(A, (W, P), GB300_PolarNewton(; maxiter, tol))
 * Replaces the reference's left_polar!(::PolarNewton) + left_polar_newton!
 * (src/implementations/polar.jl:99-111,128-166), _avgdiff! (polar.jl:209-220)
 * and project_hermitian! (src/implementations/projections.jl:61-108).
 * m >= n required.  A (m x n) is destroyed.  W: m x n.  P: n x n Hermitian,
 * or NULL (reference: empty P = not wanted, polar.jl:102-104).
 * info->iterations / residual / converged report the Newton loop; a
 * non-converged result is returned, not an error (the reference @warns,
 * polar.jl:159-161).  The host synchronizes `stream` once per Newton
 * iteration to evaluate the stopping test, like the reference's host loop.
 */
int mak_left_polar_workspace(int dtype, int64_t m, int64_t n, int want_p,
                             const mak_polar_opts* opts, size_t* bytes);
int mak_left_polar_newton_d(int64_t m, int64_t n, double* A, int64_t lda, double* W, int64_t ldw,
                            double* P, int64_t ldp, const mak_polar_opts* opts, void* work,
                            size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_left_polar_newton_z(int64_t m, int64_t n, void* A, int64_t lda, void* W, int64_t ldw,
                            void* P, int64_t ldp, const mak_polar_opts* opts, void* work,
                            size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_left_polar_newton_s(int64_t m, int64_t n, float* A, int64_t lda, float* W, int64_t ldw,
                            float* P, int64_t ldp, const mak_polar_opts* opts, void* work,
                            size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_left_polar_newton_c(int64_t m, int64_t n, void* A, int64_t lda, void* W, int64_t ldw,
                            void* P, int64_t ldp, const mak_polar_opts* opts, void* work,
                            size_t work_bytes, mak_info* info, mak_stream_t stream);

/* right_polar!(A, (P, Wh), GB300_PolarNewton(; maxiter, tol))
 * Replaces the reference's right_polar!(::PolarNewton) and
 * right_polar_newton! (src/implementations/polar.jl:113-125,168-206):
 * A = P Wh (n >= m required), computed as the conjugate transpose of the
 * left polar decomposition A^H = Wh^H P, the same Newton iteration
 * transposed.  A (m x n) is read, not destroyed.  P: m x m Hermitian, or NULL
 * (not wanted).  Wh: m x n with orthonormal rows.  info as for the left form.
 */
int mak_right_polar_workspace(int dtype, int64_t m, int64_t n, int want_p,
                              const mak_polar_opts* opts, size_t* bytes);
int mak_right_polar_newton_d(int64_t m, int64_t n, const double* A, int64_t lda, double* P,
                             int64_t ldp, double* Wh, int64_t ldwh, const mak_polar_opts* opts,
                             void* work, size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_right_polar_newton_z(int64_t m, int64_t n, const void* A, int64_t lda, void* P,
                             int64_t ldp, void* Wh, int64_t ldwh, const mak_polar_opts* opts,
                             void* work, size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_right_polar_newton_s(int64_t m, int64_t n, const float* A, int64_t lda, float* P,
                             int64_t ldp, float* Wh, int64_t ldwh, const mak_polar_opts* opts,
                             void* work, size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_right_polar_newton_c(int64_t m, int64_t n, const void* A, int64_t lda, void* P,
                             int64_t ldp, void* Wh, int64_t ldwh, const mak_polar_opts* opts,
                             void* work, size_t work_bytes, mak_info* info, mak_stream_t stream);

/* -------------------------------------------------------------- batched ---
 * Many independent, uneven blocks in one stream-ordered call (the symmetry
 * sectors of a block-sparse tensor).  The reference has no batched entry: a
 * caller loops qr_compact! / left_polar! over the blocks.  Items live in HOST
 * memory and hold DEVICE pointers; element types may be mixed.  Blocks are
 * scheduled longest-first over internal streams that fork from and join back
 * into `stream`, so the whole batch can be captured into a CUDA graph (the
 * internal streams are created by the first call, which must precede any
 * capture).  `infos` is a DEVICE array of nitems records.  Batched polar
 * launches opts->maxiter Newton iterations per block and stops each block on
 * the device once it meets the tolerance (no host synchronization);
 * infos[i].iterations is the number of steps block i took.
 */
typedef struct {
  int32_t dtype;    /* MAK_F64 / MAK_C64 / MAK_F32 / MAK_C32                 */
  int32_t reserved;
  int64_t m, n;
  void* A;          /* m x n, destroyed                                      */
  int64_t lda;
  void* Q;          /* QR: Q (m x min(m,n));  polar: W (m x n)               */
  int64_t ldq;
  void* R;          /* QR: R (min(m,n) x n);  polar: P (n x n); NULL = skip  */
  int64_t ldr;
} mak_batch_item;

int mak_batched_qr_workspace(const mak_batch_item* items, int nitems, const mak_qr_opts* opts,
                             size_t* bytes);
int mak_batched_qr_compact(const mak_batch_item* items, int nitems, const mak_qr_opts* opts,
                           void* work, size_t work_bytes, mak_info* infos, mak_stream_t stream);
int mak_batched_left_polar_workspace(const mak_batch_item* items, int nitems,
                                     const mak_polar_opts* opts, size_t* bytes);
/* Small blocks (no counterpart in the reference: qr_compact! per block,
 * src/implementations/qr.jl:132-188).  A QR block whose m x n elements (plus
 * 2 min(m,n)) fit mak_small_qr_max_bytes() bytes is factored by ONE CTA in
 * shared memory; mak_batched_qr_compact sends all such blocks of a call to
 * one persistent launch (its items copied into the launch's parameters)
 * beside the internal streams that take the larger ones.
 * mak_batched_qr_compact_device takes the work list in DEVICE memory
 * (`items`: nitems mak_batch_item records, e.g. written by a previous
 * kernel; read by the kernel, so the host never sees the shapes): every item
 * is factored by the one-CTA kernel (opts->positive honoured), and an item
 * that does not fit reports MAK_ERR_UNSUPPORTED in its record.  No
 * workspace; `infos` is a DEVICE array of nitems records.
 * mak_small_qr_max_bytes: the shared memory a block may take (the tuning
 * value MAK_SMALL_QR_BYTES, default 196 KiB, capped by the device; 0 = off). */
int mak_batched_qr_compact_device(const mak_batch_item* items, int nitems,
                                  const mak_qr_opts* opts, mak_info* infos, mak_stream_t stream);
int mak_small_qr_max_bytes(void);
/* The same for left_polar! (PolarNewton, reference
 * src/implementations/polar.jl:128-166): a block with m >= n whose m n +
 * 2 n^2 + 2 n elements and n pivot indices fit mak_small_polar_max_bytes()
 * runs the whole Newton iteration (QR of A when m > n, Gauss-Jordan inverses
 * with partial pivoting, at most opts->maxiter steps, stopped at opts->tol or
 * eps(real T)^(2/3)) in one CTA; mak_batched_left_polar sends such blocks to
 * one persistent launch, mak_batched_left_polar_device takes a DEVICE work
 * list (W in Q, P in R; infos[i].iterations / converged / singular as for a
 * single call).  MAK_SMALL_POLAR_BYTES sets the limit (default 196 KiB). */
int mak_batched_left_polar_device(const mak_batch_item* items, int nitems,
                                  const mak_polar_opts* opts, mak_info* infos,
                                  mak_stream_t stream);
int mak_small_polar_max_bytes(void);
int mak_batched_left_polar(const mak_batch_item* items, int nitems, const mak_polar_opts* opts,
                           void* work, size_t work_bytes, mak_info* infos, mak_stream_t stream);

/* Batched reverse rules over a list of blocks (the pullbacks of a whole
 * block-sparse tensor, or of every tensor of an orthogonalisation sweep, in
 * one call); no counterpart in the reference, whose callers loop
 * qr_pullback! / left_polar_pullback! (src/pullbacks/qr.jl:73-120,
 * src/pullbacks/polar.jl:7-29) over the blocks.  Items live in HOST memory
 * and hold DEVICE pointers; element types may be mixed; blocks are scheduled
 * over the same internal streams as the batched factorizations.  Each dA is
 * ACCUMULATED into; dF1 / dF2 may be NULL (a zero tangent).  `infos` is a
 * DEVICE array of nitems records.
 *  - mak_batched_qr_pullback: qr_compact factors (F1 = Q m x min(m,n),
 *    F2 = R min(m,n) x n, dF1 = dQ, dF2 = dR); the ranks of all blocks are
 *    computed first and read with ONE host synchronization of `stream`.
 *  - mak_batched_left_polar_pullback: F1 = W (m x n, m >= n), F2 = P (n x n),
 *    dF1 = dW, dF2 = dP; the Sylvester sign iteration of every block runs a
 *    fixed number of steps and stops on the device (no host
 *    synchronization); infos[i].iterations / converged report it. */
typedef struct {
  int32_t dtype;     /* MAK_F64 / MAK_C64 / MAK_F32 / MAK_C32                  */
  int32_t reserved;
  int64_t m, n;
  void* dA;          /* m x n, accumulated into                               */
  int64_t ldda;
  const void* F1;    /* Q or W                                                */
  int64_t ld1;
  const void* F2;    /* R or P                                                */
  int64_t ld2;
  const void* dF1;   /* dQ or dW, or NULL                                     */
  int64_t ldd1;
  const void* dF2;   /* dR or dP, or NULL                                     */
  int64_t ldd2;
} mak_batch_pullback_item;

int mak_batched_qr_pullback_workspace(const mak_batch_pullback_item* items, int nitems,
                                      const mak_pullback_opts* opts, size_t* bytes);
int mak_batched_qr_pullback(const mak_batch_pullback_item* items, int nitems,
                            const mak_pullback_opts* opts, void* work, size_t work_bytes,
                            mak_info* infos, mak_stream_t stream);
int mak_batched_left_polar_pullback_workspace(const mak_batch_pullback_item* items, int nitems,
                                              const mak_pullback_opts* opts, size_t* bytes);
int mak_batched_left_polar_pullback(const mak_batch_pullback_item* items, int nitems,
                                    const mak_pullback_opts* opts, void* work, size_t work_bytes,
                                    mak_info* infos, mak_stream_t stream);

/* ------------------------------------------------------------ pullbacks ---
 * qr_pullback!(dA, A, (Q, R), (dQ, dR); rank_atol, gauge_atol)
 * Replaces the reference's qr_pullback! (src/pullbacks/qr.jl:73-120) with
 * check_and_prepare_qr_cotangents (qr.jl:4-53) and qr_rank (qr.jl:1-2).
 * full = 0: Q m x min(m,n), R min(m,n) x n (qr_compact); full = 1: Q m x m,
 * R m x n (qr_full).  dA (m x n) is ACCUMULATED into (dA += ...).  dQ and/or
 * dR may be NULL (a zero tangent).  info->rank = the numerical rank p used,
 * info->gauge / gauge_atol = the gauge-dependent cotangent size and the
 * tolerance the reference warns against.  Synchronizes `stream` once (to
 * read p, which fixes the shapes of the products).
 */
int mak_qr_pullback_workspace(int dtype, int64_t m, int64_t n, int full, int precision,
                              size_t* bytes);
int mak_qr_pullback_d(int64_t m, int64_t n, int full, double* dA, int64_t ldda, const double* Q,
                      int64_t ldq, const double* R, int64_t ldr, const double* dQ, int64_t lddq,
                      const double* dR, int64_t lddr, const mak_pullback_opts* opts, void* work,
                      size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_qr_pullback_z(int64_t m, int64_t n, int full, void* dA, int64_t ldda, const void* Q,
                      int64_t ldq, const void* R, int64_t ldr, const void* dQ, int64_t lddq,
                      const void* dR, int64_t lddr, const mak_pullback_opts* opts, void* work,
                      size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_qr_pullback_s(int64_t m, int64_t n, int full, float* dA, int64_t ldda, const float* Q,
                      int64_t ldq, const float* R, int64_t ldr, const float* dQ, int64_t lddq,
                      const float* dR, int64_t lddr, const mak_pullback_opts* opts, void* work,
                      size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_qr_pullback_c(int64_t m, int64_t n, int full, void* dA, int64_t ldda, const void* Q,
                      int64_t ldq, const void* R, int64_t ldr, const void* dQ, int64_t lddq,
                      const void* dR, int64_t lddr, const mak_pullback_opts* opts, void* work,
                      size_t work_bytes, mak_info* info, mak_stream_t stream);

/* left_polar_pullback!(dA, A, (W, P), (dW, dP))
 * Replaces the reference's left_polar_pullback! (src/pullbacks/polar.jl:7-29),
 * including the Sylvester solve P C + C P = M - M^H (src/common/pullbacks.jl:15),
 * which the reference's CUDA extension runs on the host
 * (ext/MatrixAlgebraKitCUDAExt/MatrixAlgebraKitCUDAExt.jl:193-198); here it is
 * a device sign-function Newton iteration.  dA is accumulated into; dW / dP
 * may be NULL.  info->iterations = sign iterations.  Synchronizes `stream`
 * once per sign iteration (stopping test).
 */
int mak_left_polar_pullback_workspace(int dtype, int64_t m, int64_t n, int precision,
                                      size_t* bytes);
int mak_left_polar_pullback_d(int64_t m, int64_t n, double* dA, int64_t ldda, const double* W,
                              int64_t ldw, const double* P, int64_t ldp, const double* dW,
                              int64_t lddw, const double* dP, int64_t lddp,
                              const mak_pullback_opts* opts, void* work, size_t work_bytes,
                              mak_info* info, mak_stream_t stream);
int mak_left_polar_pullback_z(int64_t m, int64_t n, void* dA, int64_t ldda, const void* W,
                              int64_t ldw, const void* P, int64_t ldp, const void* dW,
                              int64_t lddw, const void* dP, int64_t lddp,
                              const mak_pullback_opts* opts, void* work, size_t work_bytes,
                              mak_info* info, mak_stream_t stream);
int mak_left_polar_pullback_s(int64_t m, int64_t n, float* dA, int64_t ldda, const float* W,
                              int64_t ldw, const float* P, int64_t ldp, const float* dW,
                              int64_t lddw, const float* dP, int64_t lddp,
                              const mak_pullback_opts* opts, void* work, size_t work_bytes,
                              mak_info* info, mak_stream_t stream);
int mak_left_polar_pullback_c(int64_t m, int64_t n, void* dA, int64_t ldda, const void* W,
                              int64_t ldw, const void* P, int64_t ldp, const void* dW,
                              int64_t lddw, const void* dP, int64_t lddp,
                              const mak_pullback_opts* opts, void* work, size_t work_bytes,
                              mak_info* info, mak_stream_t stream);

/* right_polar_pullback!(dA, A, (P, Wh), (dP, dWh))
 * Replaces the reference's right_polar_pullback! (src/pullbacks/polar.jl:
 * 37-59): computed as the conjugate transpose of the left pullback of A^H at
 * (Wh^H, P) with cotangents (dWh^H, dP), which carries the same Sylvester
 * solve on the device.  m <= n.  dA (m x n) is accumulated into; dP / dWh may
 * be NULL (a zero tangent).  Synchronizes `stream` once per sign iteration.
 */
int mak_right_polar_pullback_workspace(int dtype, int64_t m, int64_t n, int precision,
                                       size_t* bytes);
int mak_right_polar_pullback_d(int64_t m, int64_t n, double* dA, int64_t ldda, const double* P,
                               int64_t ldp, const double* Wh, int64_t ldwh, const double* dP,
                               int64_t lddp, const double* dWh, int64_t lddwh,
                               const mak_pullback_opts* opts, void* work, size_t work_bytes,
                               mak_info* info, mak_stream_t stream);
int mak_right_polar_pullback_z(int64_t m, int64_t n, void* dA, int64_t ldda, const void* P,
                               int64_t ldp, const void* Wh, int64_t ldwh, const void* dP,
                               int64_t lddp, const void* dWh, int64_t lddwh,
                               const mak_pullback_opts* opts, void* work, size_t work_bytes,
                               mak_info* info, mak_stream_t stream);
int mak_right_polar_pullback_s(int64_t m, int64_t n, float* dA, int64_t ldda, const float* P,
                               int64_t ldp, const float* Wh, int64_t ldwh, const float* dP,
                               int64_t lddp, const float* dWh, int64_t lddwh,
                               const mak_pullback_opts* opts, void* work, size_t work_bytes,
                               mak_info* info, mak_stream_t stream);
int mak_right_polar_pullback_c(int64_t m, int64_t n, void* dA, int64_t ldda, const void* P,
                               int64_t ldp, const void* Wh, int64_t ldwh, const void* dP,
                               int64_t lddp, const void* dWh, int64_t lddwh,
                               const mak_pullback_opts* opts, void* work, size_t work_bytes,
                               mak_info* info, mak_stream_t stream);

/* left_polar_pushforward!(dA, A, (W, P), (dW, dP))
 * Replaces the reference's left_polar_pushforward!
 * (src/pushforwards/polar.jl:1-12): the tangent of A = W P along dA,
 *   dP0 = W^H dA, K = sylvester(P, P, dP0^H - dP0), dW = (I - W W^H) dA P^-1
 *   + W K, dP = dP0 - K P,
 * with the Sylvester solve on the device (the pullback's sign iteration).
 * m >= n.  dW (m x n) and dP (n x n) are outputs (overwritten).
 */
int mak_left_polar_pushforward_workspace(int dtype, int64_t m, int64_t n, int precision,
                                         size_t* bytes);
int mak_left_polar_pushforward_d(int64_t m, int64_t n, const double* dA, int64_t ldda,
                                 const double* W, int64_t ldw, const double* P, int64_t ldp,
                                 double* dW, int64_t lddw, double* dP, int64_t lddp,
                                 const mak_pullback_opts* opts, void* work, size_t work_bytes,
                                 mak_info* info, mak_stream_t stream);
int mak_left_polar_pushforward_z(int64_t m, int64_t n, const void* dA, int64_t ldda,
                                 const void* W, int64_t ldw, const void* P, int64_t ldp,
                                 void* dW, int64_t lddw, void* dP, int64_t lddp,
                                 const mak_pullback_opts* opts, void* work, size_t work_bytes,
                                 mak_info* info, mak_stream_t stream);
int mak_left_polar_pushforward_s(int64_t m, int64_t n, const float* dA, int64_t ldda,
                                 const float* W, int64_t ldw, const float* P, int64_t ldp,
                                 float* dW, int64_t lddw, float* dP, int64_t lddp,
                                 const mak_pullback_opts* opts, void* work, size_t work_bytes,
                                 mak_info* info, mak_stream_t stream);
int mak_left_polar_pushforward_c(int64_t m, int64_t n, const void* dA, int64_t ldda,
                                 const void* W, int64_t ldw, const void* P, int64_t ldp,
                                 void* dW, int64_t lddw, void* dP, int64_t lddp,
                                 const mak_pullback_opts* opts, void* work, size_t work_bytes,
                                 mak_info* info, mak_stream_t stream);

/* right_polar_pushforward!(dA, A, (P, Wh), (dP, dWh))
 * Replaces the reference's right_polar_pushforward!
 * (src/pushforwards/polar.jl:14-26): the tangent of A = P Wh along dA,
 * computed as the conjugate transpose of the left pushforward of A^H at
 * (Wh^H, P) along dA^H.  m <= n.  dP (m x m) and dWh (m x n) are outputs.
 */
int mak_right_polar_pushforward_workspace(int dtype, int64_t m, int64_t n, int precision,
                                          size_t* bytes);
int mak_right_polar_pushforward_d(int64_t m, int64_t n, const double* dA, int64_t ldda,
                                  const double* P, int64_t ldp, const double* Wh, int64_t ldwh,
                                  double* dP, int64_t lddp, double* dWh, int64_t lddwh,
                                  const mak_pullback_opts* opts, void* work, size_t work_bytes,
                                  mak_info* info, mak_stream_t stream);
int mak_right_polar_pushforward_z(int64_t m, int64_t n, const void* dA, int64_t ldda,
                                  const void* P, int64_t ldp, const void* Wh, int64_t ldwh,
                                  void* dP, int64_t lddp, void* dWh, int64_t lddwh,
                                  const mak_pullback_opts* opts, void* work, size_t work_bytes,
                                  mak_info* info, mak_stream_t stream);
int mak_right_polar_pushforward_s(int64_t m, int64_t n, const float* dA, int64_t ldda,
                                  const float* P, int64_t ldp, const float* Wh, int64_t ldwh,
                                  float* dP, int64_t lddp, float* dWh, int64_t lddwh,
                                  const mak_pullback_opts* opts, void* work, size_t work_bytes,
                                  mak_info* info, mak_stream_t stream);
int mak_right_polar_pushforward_c(int64_t m, int64_t n, const void* dA, int64_t ldda,
                                  const void* P, int64_t ldp, const void* Wh, int64_t ldwh,
                                  void* dP, int64_t lddp, void* dWh, int64_t lddwh,
                                  const mak_pullback_opts* opts, void* work, size_t work_bytes,
                                  mak_info* info, mak_stream_t stream);

/* qr_null_pullback!(dA, A, N, dN; gauge_atol)
 * Replaces the reference's qr_null_pullback! (src/pullbacks/qr.jl:141-152)
 * for N = qr_null(A) (m x (m - min(m,n))): with a nonzero dN,
 * X = (dN^H Q) R^{-H} from qr_compact(A; positive = true) on the device, and
 * dA -= N X.  The gauge ||antiherm(N^H dN)||_F goes to info->gauge against
 * info->gauge_atol (opts->gauge_atol < 0: eps(max|dN|)^(3/4)); the caller
 * warns.  A is read, not written.  dN may be NULL (nothing to add).
 */
int mak_qr_null_pullback_workspace(int dtype, int64_t m, int64_t n, int precision, size_t* bytes);
int mak_qr_null_pullback_d(int64_t m, int64_t n, double* dA, int64_t ldda, const double* A,
                           int64_t lda, const double* N, int64_t ldn, const double* dN,
                           int64_t lddn, const mak_pullback_opts* opts, void* work,
                           size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_qr_null_pullback_z(int64_t m, int64_t n, void* dA, int64_t ldda, const void* A,
                           int64_t lda, const void* N, int64_t ldn, const void* dN, int64_t lddn,
                           const mak_pullback_opts* opts, void* work, size_t work_bytes,
                           mak_info* info, mak_stream_t stream);
int mak_qr_null_pullback_s(int64_t m, int64_t n, float* dA, int64_t ldda, const float* A,
                           int64_t lda, const float* N, int64_t ldn, const float* dN,
                           int64_t lddn, const mak_pullback_opts* opts, void* work,
                           size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_qr_null_pullback_c(int64_t m, int64_t n, void* dA, int64_t ldda, const void* A,
                           int64_t lda, const void* N, int64_t ldn, const void* dN, int64_t lddn,
                           const mak_pullback_opts* opts, void* work, size_t work_bytes,
                           mak_info* info, mak_stream_t stream);

/* lq_pullback!(dA, A, (L, Q), (dL, dQ); rank_atol, gauge_atol)
 * Replaces the reference's lq_pullback! (src/pullbacks/lq.jl:71-112), as the
 * conjugate transpose of qr_pullback! of A^H at (Q^H, L^H) with (dQ^H, dL^H).
 * full = 1 for lq_full output (Q n x n, L m x n; only differs when n > m).
 * dA accumulated into; dL / dQ may be NULL.  Same info fields as
 * mak_qr_pullback_*.
 */
int mak_lq_pullback_workspace(int dtype, int64_t m, int64_t n, int full, int precision,
                              size_t* bytes);
int mak_lq_pullback_d(int64_t m, int64_t n, int full, double* dA, int64_t ldda, const double* L,
                      int64_t ldl, const double* Q, int64_t ldq, const double* dL, int64_t lddl,
                      const double* dQ, int64_t lddq, const mak_pullback_opts* opts, void* work,
                      size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_lq_pullback_z(int64_t m, int64_t n, int full, void* dA, int64_t ldda, const void* L,
                      int64_t ldl, const void* Q, int64_t ldq, const void* dL, int64_t lddl,
                      const void* dQ, int64_t lddq, const mak_pullback_opts* opts, void* work,
                      size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_lq_pullback_s(int64_t m, int64_t n, int full, float* dA, int64_t ldda, const float* L,
                      int64_t ldl, const float* Q, int64_t ldq, const float* dL, int64_t lddl,
                      const float* dQ, int64_t lddq, const mak_pullback_opts* opts, void* work,
                      size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_lq_pullback_c(int64_t m, int64_t n, int full, void* dA, int64_t ldda, const void* L,
                      int64_t ldl, const void* Q, int64_t ldq, const void* dL, int64_t lddl,
                      const void* dQ, int64_t lddq, const mak_pullback_opts* opts, void* work,
                      size_t work_bytes, mak_info* info, mak_stream_t stream);

/* lq_null_pullback!(dA, A, Nh, dNh; gauge_atol)
 * Replaces the reference's lq_null_pullback! (src/pullbacks/lq.jl:133-145)
 * for Nh = lq_null(A) ((n - min(m,n)) x n): X = L^{-H} Q dNh^H, dA -= X Nh,
 * as the conjugate transpose of the QR null-space rule on A^H.
 */
int mak_lq_null_pullback_workspace(int dtype, int64_t m, int64_t n, int precision, size_t* bytes);
int mak_lq_null_pullback_d(int64_t m, int64_t n, double* dA, int64_t ldda, const double* A,
                           int64_t lda, const double* Nh, int64_t ldnh, const double* dNh,
                           int64_t lddnh, const mak_pullback_opts* opts, void* work,
                           size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_lq_null_pullback_z(int64_t m, int64_t n, void* dA, int64_t ldda, const void* A,
                           int64_t lda, const void* Nh, int64_t ldnh, const void* dNh,
                           int64_t lddnh, const mak_pullback_opts* opts, void* work,
                           size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_lq_null_pullback_s(int64_t m, int64_t n, float* dA, int64_t ldda, const float* A,
                           int64_t lda, const float* Nh, int64_t ldnh, const float* dNh,
                           int64_t lddnh, const mak_pullback_opts* opts, void* work,
                           size_t work_bytes, mak_info* info, mak_stream_t stream);
int mak_lq_null_pullback_c(int64_t m, int64_t n, void* dA, int64_t ldda, const void* A,
                           int64_t lda, const void* Nh, int64_t ldnh, const void* dNh,
                           int64_t lddnh, const mak_pullback_opts* opts, void* work,
                           size_t work_bytes, mak_info* info, mak_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* MAK_GB300_H */
