// Split-precision GEMM on the tcgen05 tensor cores (Ozaki scheme I).
//
// C = alpha * op(A) op(B) + beta * C for Float64 / ComplexF64 data, computed
// from bf16 products with fp32 accumulation in tensor memory, to an accuracy
// comparable with a native FP64 GEMM (~1e-15 relative to sum |a||b|).
//
// 1. Row exponents E_i (of op(A)) and column exponents F_j (of op(B)) over
//    the whole K range: |a_ik| < 2^E_i.
// 2. Every element is cut, with integer operations on its IEEE bits, into
//    S = 9 signed 6-bit digits of the fixed-point value a 2^(6S - E_i):
//        a = 2^(E_i - 6) sum_p d_p 2^(-6(p-1)),   |d_p| <= 63.
//    Plane p stores d_p 2^(-6(p-1)) as bf16 (exact: 6 significant bits).
//    Complex data is made real: op(A) -> [re | im] (K doubled) and
//    op(B) -> [[re, im], [-im, re]] (K and N doubled).
// 3. The tcgen05 kernel multiplies plane pairs (p, q) with p + q <= S + 1
//    (45 bf16 GEMMs per FP64 GEMM).  All products of one group d = p + q
//    carry the same scale 2^(-6(d-2)), so each exact group (d = 2..7, at
//    most 6 pairs) sums EXACTLY in its fp32 TMEM accumulator over a chunk of
//    512 of K (6 x 512 x 63^2 < 2^24); every chunk the epilogue warps convert
//    those sums to integers and add them to an int64 fixed-point accumulator
//    per output (exact).  The remaining groups d >= 8 (weight <= 2^-36)
//    share one "tail" accumulator that is never flushed.  Measured on GB300,
//    the tensor core's fp32 accumulation keeps only ~20 bits per MMA with a
//    truncation bias, so a group is either exact or lightly weighted: with
//    7-bit digits and d = 5 in the tail the product error was ~1e-11.  The
//    FP64 pipe (1 TFLOP/s on GB300) only sees a handful of operations per
//    output element in the final epilogue.
//
// Kernel shape: 128 x 64 output tile per CTA, K-step 32 (one 64-byte
// swizzled row per operand row), 2-stage TMA pipeline of S A-plane and
// S B-plane tiles per stage, warp-specialised: warp 4 issues TMA, warp 5
// issues the MMAs, warps 0-3 own TMEM lanes 0-127 for the epilogue.
// Every mbarrier wait is bounded; on timeout the CTA records
// MAK_ERR_TIMEOUT, drains its in-flight copies (bounded), frees TMEM and
// exits.  Optional split-K writes FP64 partial tiles that a reduce kernel
// folds (deterministic order).
#include <cuda.h>
#include <cuda_bf16.h>

#include <mutex>

#include "gemm.cuh"
#include "internal.h"

namespace mak {

constexpr int OZ_BM = 128, OZ_BN = 64, OZ_BK = 32;
constexpr int OZ_KSTEPS_PER_CHUNK = 16; // 512 of K between exact flushes
constexpr int OZ_BITS = 6;              // bits per digit plane
constexpr int OZ_STAGES = 2;
constexpr int OZ_THREADS = 192;         // 4 epilogue warps + TMA warp + MMA warp
constexpr int OZ_TMEM_COLS = 512;       // 7 accumulators x 64 columns (power-of-two alloc)
constexpr long long OZ_SPIN = 1ll << 26;

struct OzArgs {
  int M, Nl, nkt;           // logical output rows, logical output cols, K-steps (this split)
  int kt0;                  // first K-step of this split
  const int* EA;            // [Mpad]
  const int* EB;            // [Nlpad]
  double* C;                // output (FP64 view; complex: interleaved re/im)
  int64_t ldc;              // in elements of the data type
  int cpx;                  // complex output mapping
  int Nc;                   // complex: number of complex columns (Nl = 2 Nc)
  double alpha, beta;       // real scalars
  double* part;             // split-K partials (nullptr: write C directly)
  int64_t part_stride;      // per split
  int* status;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// tcgen05 shared-memory matrix descriptor, K-major operand, 64-byte swizzle:
// rows of 64 B, 8-row core groups 512 B apart.
__device__ __forceinline__ uint64_t oz_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;            // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(512 >> 4) << 32;   // stride byte offset
  d |= (uint64_t)1 << 46;            // descriptor version (sm_100 family)
  d |= (uint64_t)4 << 61;            // SWIZZLE_64B
  return d;
}

// instruction descriptor: bf16 x bf16 -> fp32, K-major A and B, M=128, N=64
constexpr uint32_t OZ_IDESC =
    (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(OZ_BN >> 3) << 17) | ((uint32_t)(OZ_BM >> 4) << 24);

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait; returns false (and raises the abort flag) on timeout or abort
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                          int* status) {
  long long spins = 0;
  while (!mbar_try(bar, parity)) {
    if (*abort_flag) return false;
    if (++spins > OZ_SPIN) {
      *abort_flag = 1;
      atomicExch(status, MAK_ERR_TIMEOUT);
      return false;
    }
  }
  return true;
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0,
                                            int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, "
      "%4, %5}], [%2];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}
__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t ad, uint64_t bd, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(ad), "l"(bd), "r"(OZ_IDESC), "r"(acc));
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
      smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int j = 0; j < 16; j++) v[j] = __uint_as_float(r[j]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// x * 2^e by integer arithmetic on the exponent field (ldexp outside the
// normal range)
__device__ __forceinline__ double scale_pow2(double x, int e) {
  const long long b = __double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7FF);
  if (ex == 0 || ex + e <= 0 || ex + e >= 2047) return ldexp(x, e);
  return __longlong_as_double(b + ((long long)e << 52));
}

// group accumulator of pair (p, q) (1-based digits): 0..4 exact groups d=2..6; 5 tail
constexpr int OZ_EXACT = 6;                // exact groups d = 2 .. OZ_EXACT + 1
constexpr int OZ_NGROUPS = OZ_EXACT + 1;   // + the tail
__host__ __device__ constexpr int oz_group(int p, int q) {
  return (p + q <= OZ_EXACT + 1) ? (p + q - 2) : OZ_EXACT;
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                 "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
#pragma unroll
  for (int j = 0; j < 8; j++) v[j] = __uint_as_float(r[j]);
}

template <int S>
__global__ void __launch_bounds__(OZ_THREADS, 1)
oz_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
               OzArgs a) {
  constexpr int A_TILE = OZ_BM * OZ_BK * 2;  // bytes per A-plane tile (8 KB)
  constexpr int B_TILE = OZ_BN * OZ_BK * 2;  // bytes per B-plane tile (4 KB)
  constexpr int STAGE = S * (A_TILE + B_TILE);
  extern __shared__ __align__(1024) unsigned char oz_smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)oz_smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full_bar[OZ_STAGES], empty_bar[OZ_STAGES];
  __shared__ __align__(8) uint64_t acc_full, acc_empty, drain_bar;
  __shared__ uint32_t tmem_base_s;
  __shared__ int abort_s;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * OZ_BM, n0 = blockIdx.y * OZ_BN;
  const int nkt = a.nkt;
  const int nchunks = (nkt + OZ_KSTEPS_PER_CHUNK - 1) / OZ_KSTEPS_PER_CHUNK;

  if (tid == 0) {
    abort_s = 0;
    for (int s = 0; s < OZ_STAGES; s++) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&acc_full, 1);
    mbar_init(&acc_empty, 128);
    mbar_init(&drain_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base_s)),
                 "r"(OZ_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_s;
  volatile int* abort_flag = &abort_s;

  if (warp == 4) {
    // ------------------------------------------------------------ TMA producer
    if (lane == 0) {
      int issued = 0;
      for (int kt = 0; kt < nkt; kt++) {
        const int s = kt % OZ_STAGES;
        if (kt >= OZ_STAGES) {
          if (!mbar_wait(&empty_bar[s], ((kt / OZ_STAGES) - 1) & 1, abort_flag, a.status)) break;
        }
        unsigned char* st = smem + s * STAGE;
        mbar_expect_tx(&full_bar[s], STAGE);
        const int kc = (a.kt0 + kt) * OZ_BK;
#pragma unroll
        for (int p = 0; p < S; p++) tma_load_3d(st + p * A_TILE, &tmA, &full_bar[s], kc, m0, p);
#pragma unroll
        for (int q = 0; q < S; q++)
          tma_load_3d(st + S * A_TILE + q * B_TILE, &tmB, &full_bar[s], kc, n0, q);
        issued = kt + 1;
      }
      // drain: every issued stage must have landed before the CTA can exit
      for (int kt = (issued > OZ_STAGES ? issued - OZ_STAGES : 0); kt < issued; kt++) {
        long long spins = 0;
        while (!mbar_try(&full_bar[kt % OZ_STAGES], (kt / OZ_STAGES) & 1) && ++spins < OZ_SPIN) {
        }
      }
    }
  } else if (warp == 5) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      bool tail_started = false;
      for (int kt = 0; kt < nkt; kt++) {
        const int s = kt % OZ_STAGES;
        const int chunk = kt / OZ_KSTEPS_PER_CHUNK;
        const bool chunk_first = (kt % OZ_KSTEPS_PER_CHUNK) == 0;
        if (chunk_first && chunk > 0) {
          if (!mbar_wait(&acc_empty, (chunk - 1) & 1, abort_flag, a.status)) break;
        }
        if (!mbar_wait(&full_bar[s], (kt / OZ_STAGES) & 1, abort_flag, a.status)) break;
        tc_fence_after();
        const uint32_t sa = smem_u32(smem + s * STAGE);
        const uint32_t sb = sa + S * A_TILE;
        bool first_in_group[OZ_NGROUPS];
#pragma unroll
        for (int g = 0; g < OZ_EXACT; g++) first_in_group[g] = chunk_first;
        first_in_group[OZ_EXACT] = !tail_started;
#pragma unroll
        for (int d = 2; d <= S + 1; d++) {
#pragma unroll
          for (int p = 1; p < d; p++) {
            const int q = d - p;
            if (p > S || q > S) continue;
            const int g = oz_group(p, q);
#pragma unroll
            for (int ks = 0; ks < 2; ks++) {
              const uint64_t ad = oz_desc(sa + (p - 1) * A_TILE + ks * 32);
              const uint64_t bd = oz_desc(sb + (q - 1) * B_TILE + ks * 32);
              umma(tmem + g * OZ_BN, ad, bd, first_in_group[g] ? 0u : 1u);
              first_in_group[g] = false;
            }
          }
        }
        tail_started = true;
        umma_commit(&empty_bar[s]);
        const bool chunk_last = ((kt + 1) % OZ_KSTEPS_PER_CHUNK) == 0 || kt + 1 == nkt;
        if (chunk_last) umma_commit(&acc_full);
      }
      // every MMA issued must have completed before TMEM is released
      umma_commit(&drain_bar);
      long long spins = 0;
      while (!mbar_try(&drain_bar, 0) && ++spins < OZ_SPIN) {
      }
    }
  } else {
    // ------------------------------------------------------------ epilogue warps 0-3
    const int r = warp * 32 + lane;  // tile row == TMEM lane
    const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
    long long acc[OZ_BN];
#pragma unroll
    for (int c = 0; c < OZ_BN; c++) acc[c] = 0;
    bool ok = true;
    for (int chunk = 0; chunk < nchunks && ok; chunk++) {
      ok = mbar_wait(&acc_full, chunk & 1, abort_flag, a.status);
      if (!ok) break;
      tc_fence_after();
#pragma unroll
      for (int c0 = 0; c0 < OZ_BN; c0 += 8) {
        float s[OZ_EXACT][8];
#pragma unroll
        for (int g = 0; g < OZ_EXACT; g++) tmem_ld8(lane_addr + g * OZ_BN + c0, s[g]);
        tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 8; j++) {
          // group d holds an integer times 2^(-6(d-2)) below 2^24: convert
          // each exactly and sum in units of 2^(-6(OZ_EXACT-1)) of the
          // group-2 scale
          long long t = 0;
#pragma unroll
          for (int g = 0; g < OZ_EXACT; g++)
            t += (long long)__float2int_rn(s[g][j] * (float)(1 << (OZ_BITS * g)))
                 << (OZ_BITS * (OZ_EXACT - 1 - g));
          acc[c0 + j] += t;
        }
      }
      tc_fence_before();
      mbar_arrive(&acc_empty);
    }
    if (ok) {
      // final: value = 2^(E+F-12-SH) (acc + tail 2^SH), SH = 6(OZ_EXACT-1).
      // The FP64 pipe is 1/1900 of the tensor rate, so each output costs two
      // conversions and two FP64 FMAs; the scale alpha 2^e is built by
      // integer exponent arithmetic.
      constexpr int SH = OZ_BITS * (OZ_EXACT - 1);
      const int gi = m0 + r;
      const int Ei = (gi < a.M) ? a.EA[gi] : 0;
      const double mult = a.part ? 1.0 : a.alpha;
      const bool beta0 = a.part != nullptr || a.beta == 0.0, beta1 = a.beta == 1.0;
#pragma unroll
      for (int c0 = 0; c0 < OZ_BN; c0 += 16) {
        float tl[16];
        tmem_ld16(lane_addr + OZ_EXACT * OZ_BN + c0, tl);
        tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 16; j++) {
          const int gj = n0 + c0 + j;
          if (gi >= a.M || gj >= a.Nl) continue;
          // the tail carries bits below the 2^-SH unit of acc: add it in FP64
          const double v = fma((double)tl[j], (double)(1ll << SH), (double)acc[c0 + j]);
          const double sc = scale_pow2(mult, Ei + a.EB[gj] - 2 * OZ_BITS - SH);
          if (a.part) {
            a.part[(int64_t)gj * a.M + gi] = v * sc;  // split-K partial, ld = M
            continue;
          }
          double* dst;
          if (a.cpx) {
            const int jc = gj < a.Nc ? gj : gj - a.Nc;
            dst = a.C + 2 * ((int64_t)gi + (int64_t)jc * a.ldc) + (gj < a.Nc ? 0 : 1);
          } else {
            dst = a.C + (int64_t)gi + (int64_t)gj * a.ldc;
          }
          *dst = beta0 ? v * sc : (beta1 ? fma(v, sc, *dst) : fma(v, sc, a.beta * *dst));
        }
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(OZ_TMEM_COLS));
  }
}

// split-K fold: C = alpha * sum_s part[s] + beta * C  (fixed order)
__global__ void oz_reduce_kernel(int M, int Nl, int splits, const double* part, int64_t stride,
                                 double* C, int64_t ldc, int cpx, int Nc, double alpha,
                                 double beta) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)M * Nl) return;
  const int gi = (int)(e % M), gj = (int)(e / M);
  double v = 0.0;
  for (int s = 0; s < splits; s++) v += part[s * stride + e];
  double* dst;
  if (cpx) {
    const int jc = gj < Nc ? gj : gj - Nc;
    dst = C + 2 * ((int64_t)gi + (int64_t)jc * ldc) + (gj < Nc ? 0 : 1);
  } else {
    dst = C + (int64_t)gi + (int64_t)gj * ldc;
  }
  double out = alpha * v;
  if (beta != 0.0) out = fma(beta, *dst, out);
  *dst = out;
}

// ---------------------------------------------------------------- splitting --
// Logical real operand X (R x K) built from op(A) (A side) or op(B)^T (B side),
// with the complex-to-real mapping described at the top of the file.
template <class T>
struct OzSrc {
  Operand<T> op;
  int side;   // 0: A side (rows of op(A)), 1: B side (columns of op(B))
  int M0, K0; // underlying op(A) rows / op(B) cols, and K
};

template <class T>
__device__ __forceinline__ double oz_fetch(const OzSrc<T>& s, int r, int k) {
  if constexpr (!traits<T>::cpx) {
    T v = (s.side == 0) ? load_op(s.op, r, k) : load_op(s.op, k, r);
    return (double)v;
  } else {
    if (s.side == 0) {
      const bool im = k >= s.K0;
      T v = load_op(s.op, r, im ? k - s.K0 : k);
      return im ? (double)v.im : (double)v.re;
    } else {
      const bool hiN = r >= s.M0, hiK = k >= s.K0;
      T v = load_op(s.op, hiK ? k - s.K0 : k, hiN ? r - s.M0 : r);
      if (!hiN) return hiK ? -(double)v.im : (double)v.re;
      return hiK ? (double)v.re : (double)v.im;
    }
  }
}

// memory-contiguous direction of the logical operand: true = along r
template <class T>
__host__ __device__ inline bool oz_contig_r(const OzSrc<T>& s) {
  return (s.side == 0) ? (s.op.op == OP_N) : (s.op.op != OP_N);
}

__device__ __forceinline__ unsigned long long absbits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}
__device__ __forceinline__ int exp_of_absbits(unsigned long long b) {
  // smallest e with |x| < 2^e (frexp exponent); 0 for x == 0
  if (b == 0) return 0;
  int ex = (int)(b >> 52);
  if (ex == 0) return -1021;  // subnormal
  return ex - 1022;
}

// Row maxima of |X| as IEEE bit patterns (non-negative doubles order like
// their bits), accumulated with atomicMax over a 2-D grid of (rows, K
// chunks) so that tall K ranges are read by many CTAs in parallel.
constexpr int OZ_EXP_KCHUNK = 1024;
template <class T>
__global__ void __launch_bounds__(256) oz_absmax_kernel(OzSrc<T> s, int R, int K,
                                                        unsigned long long* mx_bits) {
  const int k0 = blockIdx.y * OZ_EXP_KCHUNK;
  const int k1 = min(K, k0 + OZ_EXP_KCHUNK);
  if (oz_contig_r(s)) {
    // 256 consecutive rows per CTA, each thread walks the chunk of K
    const int r = blockIdx.x * 256 + threadIdx.x;
    if (r >= R) return;
    unsigned long long mx = 0;
    for (int k = k0; k < k1; k++) {
      const unsigned long long b = absbits(oz_fetch(s, r, k));
      mx = b > mx ? b : mx;
    }
    if (mx) atomicMax(&mx_bits[r], mx);
  } else {
    // 8 rows per CTA, one warp per row, lanes along K
    const int r = blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (r >= R) return;
    unsigned long long mx = 0;
    for (int k = k0 + lane; k < k1; k += 32) {
      const unsigned long long b = absbits(oz_fetch(s, r, k));
      mx = b > mx ? b : mx;
    }
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) {
      unsigned long long o = __shfl_xor_sync(0xffffffffu, mx, m);
      mx = o > mx ? o : mx;
    }
    if (lane == 0 && mx) atomicMax(&mx_bits[r], mx);
  }
}
__global__ void oz_exp_from_bits_kernel(int R, const unsigned long long* mx_bits, int* E) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < R) E[r] = exp_of_absbits(mx_bits[r]);
}
template <class T>
static int oz_exponents(cudaStream_t st, const OzSrc<T>& s, int R, int K, unsigned long long* bits,
                        int* E) {
  MAK_CUDA_TRY(cudaMemsetAsync(bits, 0, (size_t)R * sizeof(unsigned long long), st));
  const unsigned gy = (unsigned)ceil_div(K > 0 ? K : 1, OZ_EXP_KCHUNK);
  const unsigned gx = (unsigned)(oz_contig_r(s) ? ceil_div(R, 256) : ceil_div(R, 8));
  note_launch();
  oz_absmax_kernel<T><<<dim3(gx, gy), 256, 0, st>>>(s, R, K, bits);
  note_launch();
  oz_exp_from_bits_kernel<<<(unsigned)ceil_div(R, 256), 256, 0, st>>>(R, bits, E);
  return cudaGetLastError() == cudaSuccess ? 0 : MAK_ERR_CUDA;
}

// planes[p][r][k] (Rpad x Kpad, bf16) = sign * digit_p * 2^(-7(p-1)), zero padded
template <class T, int S>
__global__ void __launch_bounds__(256) oz_split_kernel(OzSrc<T> s, int R, int K, int Rpad,
                                                       int Kpad, const int* E,
                                                       __nv_bfloat16* planes) {
  __shared__ double tile[64][65];
  const int r0 = blockIdx.y * 64, k0 = blockIdx.x * 64;
  const int tid = threadIdx.x;
  const bool cr = oz_contig_r(s);
  for (int e = tid; e < 64 * 64; e += 256) {
    int rr, kk;
    if (cr) { rr = e % 64; kk = e / 64; } else { kk = e % 64; rr = e / 64; }
    const int r = r0 + rr, k = k0 + kk;
    tile[rr][kk] = (r < R && k < K) ? oz_fetch(s, r, k) : 0.0;
  }
  __syncthreads();
  constexpr int FB = OZ_BITS * S;  // fractional bits of the fixed-point value
  constexpr uint32_t DMASK = (1u << OZ_BITS) - 1u;
  const size_t plane_stride = (size_t)Rpad * Kpad;
  // each thread: one row, a pair of adjacent k
  for (int e = tid; e < 64 * 32; e += 256) {
    const int rr = e / 32, kp = (e % 32) * 2;
    const int r = r0 + rr;
    if (r >= Rpad) continue;
    const int Er = (r < R) ? E[r] : 0;
    uint32_t dig[2][S];
    bool neg[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const double x = tile[rr][kp + h];
      const unsigned long long b = (unsigned long long)__double_as_longlong(x);
      neg[h] = (b >> 63) != 0;
      int ex = (int)((b >> 52) & 0x7FF);
      unsigned long long m = b & 0x000FFFFFFFFFFFFFull;
      if (ex == 0) ex = 1; else m |= 0x0010000000000000ull;
      const int sh = ex - 1075 + FB - Er;
      unsigned long long f;
      if ((b & 0x7FFFFFFFFFFFFFFFull) == 0) f = 0;
      else if (sh >= 0) f = (sh >= 11) ? 0 : (m << sh);  // |x| < 2^E keeps f < 2^FB
      else f = (-sh >= 64) ? 0 : (m >> (-sh));
#pragma unroll
      for (int p = 0; p < S; p++)
        dig[h][p] = (uint32_t)((f >> (FB - OZ_BITS * (p + 1))) & DMASK);
    }
#pragma unroll
    for (int p = 0; p < S; p++) {
      const float sc = __int_as_float((127 - OZ_BITS * p) << 23);  // 2^(-6p)
      __nv_bfloat162 v;
      v.x = __float2bfloat16_rn((neg[0] ? -1.0f : 1.0f) * (float)dig[0][p] * sc);
      v.y = __float2bfloat16_rn((neg[1] ? -1.0f : 1.0f) * (float)dig[1][p] * sc);
      const int k = k0 + kp;
      if (k < Kpad)
        *reinterpret_cast<__nv_bfloat162*>(planes + p * plane_stride + (size_t)r * Kpad + k) = v;
    }
  }
}

// ---------------------------------------------------------------- host side --
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag f;
  std::call_once(f, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  });
  return fn;
}

static int make_plane_map(CUtensorMap* map, void* base, int S, int rows_pad, int kpad, int box_rows) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return MAK_ERR_CUDA;
  cuuint64_t dims[3] = {(cuuint64_t)kpad, (cuuint64_t)rows_pad, (cuuint64_t)S};
  cuuint64_t strides[2] = {(cuuint64_t)kpad * 2, (cuuint64_t)rows_pad * kpad * 2};
  cuuint32_t box[3] = {(cuuint32_t)OZ_BK, (cuuint32_t)box_rows, 1};
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : MAK_ERR_CUDA;
}

template <int S>
static size_t oz_smem_bytes() {
  return (size_t)OZ_STAGES * S * (OZ_BM * OZ_BK * 2 + OZ_BN * OZ_BK * 2) + 1024;
}

template <int S>
static void oz_set_attr() {
  static std::once_flag f;
  std::call_once(f, [] {
    cudaFuncSetAttribute(oz_gemm_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)oz_smem_bytes<S>());
  });
}

// slices: 9 (54-bit fixed point) for Float64 data, 5 (30-bit) for Float32 data
template <class T>
constexpr int oz_slices() { return sizeof(real_t<T>) == 8 ? 9 : 5; }

template <class T>
int oz_gemm(cudaStream_t st, int64_t M, int64_t N, int64_t K, T alpha, Operand<T> A, Operand<T> B,
            T beta, T* C, int64_t ldc, Arena& ar, int* status) {
  constexpr bool cpx = traits<T>::cpx;
  constexpr int S = oz_slices<T>();
  const int64_t Kl = cpx ? 2 * K : K;       // logical K
  const int64_t Nl = cpx ? 2 * N : N;       // logical output columns
  const int64_t Mpad = ceil_div(M > 0 ? M : 1, OZ_BM) * OZ_BM;
  const int64_t Npad = ceil_div(Nl > 0 ? Nl : 1, OZ_BN) * OZ_BN;
  const int64_t Kpad = ceil_div(Kl > 0 ? Kl : 1, OZ_BK) * OZ_BK;
  const int64_t nkt_total = Kpad / OZ_BK;
  const int64_t tiles = (Mpad / OZ_BM) * (Npad / OZ_BN);
  // split K so that about two waves of CTAs cover the SMs, whole chunks per split
  int splits = 1;
  {
    const int sms = num_sms();
    const int64_t nchunk = ceil_div(nkt_total, OZ_KSTEPS_PER_CHUNK);
    if (tiles < sms) {
      splits = (int)ceil_div(sms, tiles);
      if (splits > nchunk) splits = (int)nchunk;
      if (splits > 32) splits = 32;
      if (splits < 1) splits = 1;
    }
  }
  const int64_t chunks_per_split =
      ceil_div(ceil_div(nkt_total, OZ_KSTEPS_PER_CHUNK), splits);
  splits = (int)ceil_div(ceil_div(nkt_total, OZ_KSTEPS_PER_CHUNK), chunks_per_split);

  int* EA = ar.take<int>(Mpad);
  int* EB = ar.take<int>(Npad);
  unsigned long long* bitsA = ar.take<unsigned long long>(Mpad);
  unsigned long long* bitsB = ar.take<unsigned long long>(Npad);
  __nv_bfloat16* PA = ar.take<__nv_bfloat16>((size_t)S * Mpad * Kpad);
  __nv_bfloat16* PB = ar.take<__nv_bfloat16>((size_t)S * Npad * Kpad);
  double* part = splits > 1 ? ar.take<double>((size_t)splits * M * Nl) : nullptr;
  if (ar.base == nullptr) return 0;
  if (!ar.ok()) return MAK_ERR_WORKSPACE;
  if (M <= 0 || N <= 0) return 0;

  OzSrc<T> sa{A, 0, (int)M, (int)K};
  OzSrc<T> sb{B, 1, (int)N, (int)K};
  MAK_TRY(oz_exponents<T>(st, sa, (int)M, (int)Kl, bitsA, EA));
  MAK_TRY(oz_exponents<T>(st, sb, (int)Nl, (int)Kl, bitsB, EB));
  note_launch();
  oz_split_kernel<T, S><<<dim3((unsigned)(Kpad / 64 + (Kpad % 64 ? 1 : 0)), (unsigned)(Mpad / 64)),
                          256, 0, st>>>(sa, (int)M, (int)Kl, (int)Mpad, (int)Kpad, EA, PA);
  note_launch();
  oz_split_kernel<T, S><<<dim3((unsigned)(Kpad / 64 + (Kpad % 64 ? 1 : 0)), (unsigned)(Npad / 64)),
                          256, 0, st>>>(sb, (int)Nl, (int)Kl, (int)Npad, (int)Kpad, EB, PB);
  MAK_CUDA_TRY(cudaGetLastError());

  CUtensorMap mapA, mapB;
  MAK_TRY(make_plane_map(&mapA, PA, S, (int)Mpad, (int)Kpad, OZ_BM));
  MAK_TRY(make_plane_map(&mapB, PB, S, (int)Npad, (int)Kpad, OZ_BN));
  oz_set_attr<S>();

  const double ar_ = re_(alpha), br_ = re_(beta);
  const double work = (cpx ? 8.0 : 2.0) * (double)M * N * K;
  ProfScope prof(st, PROF_GEMM_MIXED, work);
  for (int sp = 0; sp < splits; sp++) {
    const int64_t kt0 = sp * chunks_per_split * OZ_KSTEPS_PER_CHUNK;
    int64_t nkt = chunks_per_split * OZ_KSTEPS_PER_CHUNK;
    if (kt0 + nkt > nkt_total) nkt = nkt_total - kt0;
    OzArgs args{(int)M, (int)Nl, (int)nkt, (int)kt0, EA, EB, (double*)C, ldc, cpx ? 1 : 0,
                (int)N, ar_, br_, part ? part + (size_t)sp * M * Nl : nullptr, 0,
                status};
    note_launch();
    oz_gemm_kernel<S><<<dim3((unsigned)(Mpad / OZ_BM), (unsigned)(Npad / OZ_BN)), OZ_THREADS,
                        oz_smem_bytes<S>(), st>>>(mapA, mapB, args);
    MAK_CUDA_TRY(cudaGetLastError());
  }
  if (part) {
    note_launch();
    oz_reduce_kernel<<<(unsigned)ceil_div(M * Nl, 256), 256, 0, st>>>(
        (int)M, (int)Nl, splits, part, M * Nl, (double*)C, ldc, cpx ? 1 : 0, (int)N, ar_, br_);
    MAK_CUDA_TRY(cudaGetLastError());
  }
  return 0;
}

#define MAK_INST_OZ(T)                                                                        \
  template int oz_gemm<T>(cudaStream_t, int64_t, int64_t, int64_t, T, Operand<T>, Operand<T>, \
                          T, T*, int64_t, Arena&, int*);
MAK_INST_OZ(double)
MAK_INST_OZ(zcomplex)

}  // namespace mak
