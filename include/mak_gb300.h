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
  int32_t blocksize; /* 0: library default panel width; else 1..64           */
  int32_t precision; /* MAK_PREC_NATIVE or MAK_PREC_MIXED                     */
  int32_t reserved;
} mak_qr_opts;

/* Options of PolarNewton(; maxiter, tol) (reference
 * src/implementations/polar.jl:128). */
typedef struct {
  int32_t maxiter;   /* reference default 10                                  */
  int32_t precision; /* MAK_PREC_NATIVE or MAK_PREC_MIXED                     */
  double tol;        /* <= 0: reference default eps(real T)^(2/3)             */
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

#ifdef __cplusplus
}
#endif
#endif /* MAK_GB300_H */
