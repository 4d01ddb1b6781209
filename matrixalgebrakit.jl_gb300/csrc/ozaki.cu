// Split-precision GEMM on the tcgen05 tensor cores (Ozaki scheme I).
//
// C = alpha * op(A) op(B) + beta * C for Float64 / ComplexF64 data, computed
// from bf16 products with fp32 accumulation in tensor memory, to an accuracy
// comparable with a native FP64 GEMM (~1e-15 relative to sum |a||b|).
//
// 1. Row exponents E_i (of op(A)) and column exponents F_j (of op(B)) over
//    the whole K range: |a_ik| < 2^E_i.
// 2. Every element is rounded to the 56-bit fixed-point grid of the frame
//    2^(E_i + 1) (one bit of headroom) and cut, with integer operations on
//    its IEEE bits, into S = 8 balanced 7-bit digits:
//        a = 2^(E_i + 1) sum_p d_p 2^(-7p),   |d_p| <= 64.
//    Plane p stores d_p 2^(-7(p-1)) as bf16 (exact: 7 significant bits).
//    Complex data is made real: op(A) -> [re | im] (K doubled) and
//    op(B) -> [[re, im], [-im, re]] (K and N doubled).
// 3. The tcgen05 kernel multiplies plane pairs (p, q) with p + q <= S + 1
//    (36 bf16 GEMMs per FP64 GEMM); the dropped pairs weigh <= 2^-58 of
//    2^(E_i + F_j + 2) each.  All products of one group d = p + q carry the
//    same scale 2^(-7(d-2)) and every group has its own fp32 TMEM
//    accumulator (8 groups x 64 columns = the 512 TMEM columns).  A group
//    has at most S = 8 pairs, so over a chunk of 512 of K its partial sums
//    are integers (in its scale) of magnitude <= 8 x 512 x 64^2 = 2^24:
//    exactly representable, so the tensor core's fp32 accumulation is
//    EXACT (measured on GB300: fp32 accumulation is exact whenever the
//    result is representable, and truncating otherwise, so inexact groups
//    lose precision with a bias).  Every chunk the epilogue warps convert
//    the group sums to integers and add them to a 92-bit fixed-point
//    accumulator per output (int64 high part in units of 2^-21 of the
//    group-2 scale, 28-bit low part below it): exact.  The final value is
//    rounded once to FP64 by integer operations on its bits; the FP64 pipe
//    (about 1.6 operations per clock per SM on GB300) only sees the
//    beta * C update.
//
// Kernel shape: persistent grid (one CTA per SM, each looping over output
// tiles and K splits), 128 x 64 output tile, K-step 16 (one 32-byte
// swizzled row per operand row), 4-stage TMA pipeline of S A-plane and S
// B-plane tiles per stage, warp-specialised: warp 8 issues TMA, warp 9
// issues the MMAs, warps 0-7 run the epilogue (warp w owns TMEM lanes
// 32 (w mod 4) .. +31 and output columns 32 (w div 4) .. +31).  The
// epilogue releases the accumulators before its final FP64 assembly and C
// update, so the next tile's MMAs overlap them.
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

// K per pipeline stage (16: 32-byte swizzled rows, 32: 64-byte rows) and
// the number of stages; MAK_OZ_BK / MAK_OZ_STAGES select another tiling at
// build time (the shared memory of all stages must stay within 227 KB)
#ifndef MAK_OZ_BK
#define MAK_OZ_BK 16
#endif
#ifndef MAK_OZ_STAGES
#define MAK_OZ_STAGES 4
#endif
constexpr int OZ_BM = 128, OZ_BN = 64, OZ_BK = MAK_OZ_BK;
static_assert(OZ_BK == 16 || OZ_BK == 32, "K step of 16 or 32");
constexpr int OZ_KSTEPS_PER_CHUNK = 512 / OZ_BK;  // 512 of K between exact flushes
constexpr int OZ_SMALL_CHUNK = 128 / OZ_BK;       // K <= 128: one short exact chunk
constexpr int OZ_ROW_BYTES = OZ_BK * 2;           // one swizzled K row of a plane tile
constexpr int OZ_BITS = 7;              // bits per (balanced) digit plane
constexpr int OZ_STAGES = MAK_OZ_STAGES;  // 4 x 48 KB (K step 16): finer stages keep more loads in flight
constexpr int OZ_EPI_WARPS = 8;         // two warps per TMEM lane quadrant
constexpr int OZ_THREADS = 32 * (OZ_EPI_WARPS + 2);  // + TMA warp + MMA warp
constexpr int OZ_TMA_WARP = OZ_EPI_WARPS, OZ_MMA_WARP = OZ_EPI_WARPS + 1;
constexpr int OZ_TMEM_COLS = 512;       // S group accumulators x BN columns, per buffer
constexpr long long OZ_SPIN = 1ll << 26;

// Row (column) exponents of the operands are kept as the IEEE bit patterns
// of the largest magnitudes and decoded where they are used.
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

struct OzArgs {
  int M, Nl, nkt_total;     // logical output rows, logical output cols, K-steps in all
  int split_steps;          // K-steps per split; split z starts at K-step z * split_steps
  int tiles_m, tiles_n;     // output tiles (OZ_BM x BN) along M and N
  int splits;               // K splits; work items = tiles_m * tiles_n * splits
  const unsigned long long* bitsA;  // [Mpad] largest |A| of each row, as IEEE bits
  const unsigned long long* bitsB;  // [Nlpad] largest |B| of each column
  double* C;                // output (FP64 view; complex: interleaved re/im)
  int64_t ldc;              // in elements of the data type
  int cpx;                  // complex output mapping
  int Nc;                   // complex: number of complex columns (Nl = 2 Nc)
  double alpha, beta;       // real scalars
  double* part;             // split-K partials (nullptr: write C directly), split z at
  int64_t part_stride;      //   part + z * part_stride
  int* status;
  const int* skip;          // device stop flag of a fixed-iteration loop (or nullptr)
  int merged;               // 1: one MMA per A plane and up to four B planes
};

// One work item of the persistent loop: an output tile and a K range.
// Items are numbered tile-major (M fastest, so consecutive CTAs share the
// B-plane tile in L2), then split.
struct OzWork {
  int m0, n0, kt0, nkt;
  double* part;
};
__device__ __forceinline__ OzWork oz_work(const OzArgs& a, int w, int bn) {
  const int tiles = a.tiles_m * a.tiles_n;
  const int z = w / tiles, t = w - z * tiles;
  OzWork o;
  o.m0 = (t % a.tiles_m) * OZ_BM;
  o.n0 = (t / a.tiles_m) * bn;
  o.kt0 = z * a.split_steps;
  o.nkt = min(a.nkt_total - o.kt0, a.split_steps);
  o.part = a.part ? a.part + (int64_t)z * a.part_stride : nullptr;
  return o;
}


__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// tcgen05 shared-memory matrix descriptor, K-major operand swizzled by the
// row width (32-byte rows: SWIZZLE_32B, 64-byte rows: SWIZZLE_64B), 8-row
// core groups 8 rows apart.
constexpr uint64_t oz_swizzle_code() { return OZ_ROW_BYTES == 32 ? 6 : (OZ_ROW_BYTES == 64 ? 4 : 2); }
__device__ __forceinline__ uint64_t oz_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;                             // leading byte offset (unused when swizzled)
  d |= (uint64_t)((8 * OZ_ROW_BYTES) >> 4) << 32;     // stride byte offset: 8 rows
  d |= (uint64_t)1 << 46;                             // descriptor version (sm_100 family)
  d |= oz_swizzle_code() << 61;
  return d;
}

// instruction descriptor: bf16 x bf16 -> fp32, K-major A and B, M=128, N
// columns (a multiple of 16 up to 256)
constexpr uint32_t oz_idesc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(OZ_BM >> 4) << 24);
}
constexpr uint32_t OZ_IDESC = oz_idesc(OZ_BN);

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
// the same wait for the epilogue warps, which wait microseconds for an
// accumulator chunk: a short sleep between polls leaves the issue slots of
// their SM sub-partitions to the TMA and MMA warps
__device__ __forceinline__ bool mbar_wait_backoff(uint64_t* bar, uint32_t parity,
                                                  volatile int* abort_flag, int* status) {
  long long spins = 0;
  while (!mbar_try(bar, parity)) {
    if (*abort_flag) return false;
    if (++spins > OZ_SPIN) {
      *abort_flag = 1;
      atomicExch(status, MAK_ERR_TIMEOUT);
      return false;
    }
    __nanosleep(100);
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
__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t ad, uint64_t bd, uint32_t acc,
                                     uint32_t idesc = OZ_IDESC) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
      smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// The double nearest to (-1)^flip (hi 2^lob + lo) 2^e2 (hi signed,
// 0 <= lo < 2^lob, lob <= 63), rounded to nearest even, built with integer
// operations on the 128-bit two's-complement value: GB300 issues about 1.6
// FP64 operations per clock per SM, so the conversion, the scaling and the
// sign of alpha stay off the FP64 pipe.  Results beyond the largest double
// become +-inf; results below the normal range are truncated to a subnormal
// (an absolute error below 2^-1074).
__device__ __forceinline__ double fx_to_double(long long hi, unsigned long long lo, int lob,
                                               int e2, bool flip) {
  unsigned long long xl = ((unsigned long long)hi << lob) | lo;
  unsigned long long xh = (unsigned long long)(hi >> (64 - lob));
  bool neg = (long long)xh < 0;
  if (neg) {
    xl = ~xl + 1ull;
    xh = ~xh + (xl == 0ull ? 1ull : 0ull);
  }
  if ((xh | xl) == 0ull) return 0.0;
  neg = neg != flip;
  const int lz = xh ? __clzll((long long)xh) : 64 + __clzll((long long)xl);
  unsigned long long nh, nl;
  if (lz >= 64) {
    nh = xl << (lz - 64);
    nl = 0ull;
  } else if (lz == 0) {
    nh = xh;
    nl = xl;
  } else {
    nh = (xh << lz) | (xl >> (64 - lz));
    nl = xl << lz;
  }
  unsigned long long mant = nh >> 11;  // 53 bits, leading one at bit 52
  const unsigned long long rem = nh & 0x7FFull;
  if (rem > 0x400ull || (rem == 0x400ull && (nl != 0ull || (mant & 1ull)))) mant += 1ull;
  int ex = 127 - lz + e2;  // value = mant 2^(ex - 52)
  if (mant >> 53) {
    mant >>= 1;
    ex += 1;
  }
  const unsigned long long sgn = neg ? 0x8000000000000000ull : 0ull;
  int biased = ex + 1023;
  unsigned long long bits;
  if (biased >= 2047) {
    bits = sgn | 0x7FF0000000000000ull;
  } else if (biased <= 0) {
    const int sh = 1 - biased;  // subnormal: exponent field 0, mantissa shifted
    bits = sgn | (sh >= 53 ? 0ull : (mant >> sh));
  } else {
    bits = sgn | ((unsigned long long)biased << 52) | (mant & 0x000FFFFFFFFFFFFFull);
  }
  return __longlong_as_double((long long)bits);
}

// The integer k of a group sum s = k 2^(-7g) with |k| <= 2^22: s 2^(7g) + 1.5
// 2^23 is exact in fp32 (an integer in [2^23, 2^24]), so one FFMA and one
// integer subtraction recover k.
__device__ __forceinline__ int group_int_small(float s, int g) {
  return __float_as_int(fmaf(s, __int_as_float((127 + OZ_BITS * g) << 23), 12582912.0f)) -
         0x4B400000;
}

// The integer k of a group sum s = k 2^(-7g) (|k| <= 2^24, so s is exact in
// fp32 and normal or zero), read from the IEEE bits on the integer pipe.
__device__ __forceinline__ long long group_int(float s, int g) {
  const unsigned u = __float_as_uint(s);
  const int e = (int)((u >> 23) & 0xFFu);
  const int m = (int)((u & 0x7FFFFFu) | 0x800000u);
  const int sh = e - 150 + OZ_BITS * g;  // k = m 2^sh, sh in [-23, 1] for k != 0
  int k = sh >= 0 ? (m << sh) : (m >> (-sh));
  k = e == 0 ? 0 : k;
  return (long long)((u >> 31) ? -k : k);
}

// frame of the digits: |x| < 2^(E + OZ_HEADROOM) for the row exponent E, so
// that the rounded 56-bit fixed-point value stays <= 2^55 and the leading
// balanced digit <= 64
constexpr int OZ_HEADROOM = 1;
__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float* v) {
  uint32_t r[4];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr));
#pragma unroll
  for (int j = 0; j < 4; j++) v[j] = __uint_as_float(r[j]);
}

// address of output (gi, gj) of the logical real product (complex: column
// gj < Nc is the real part of complex column gj, else the imaginary part of
// column gj - Nc)
__device__ __forceinline__ double* oz_out_ptr(double* C, int64_t ldc, int cpx, int Nc, int gi,
                                              int gj) {
  if (cpx) {
    const int jc = gj < Nc ? gj : gj - Nc;
    return C + 2 * ((int64_t)gi + (int64_t)jc * ldc) + (gj < Nc ? 0 : 1);
  }
  return C + (int64_t)gi + (int64_t)gj * ldc;
}

// CHUNK = K-steps per exact accumulator chunk: 32 (512 of K, group sums up
// to 2^24, converted from their bits) or 8 (128 of K, group sums up to 2^22,
// converted with one FFMA; products with K <= 128 use this variant).
// BN = output tile width: 64, or 32 with two accumulator buffers in TMEM
// (S x 32 columns each) so that the MMAs of the next tile run while the
// epilogue reads the previous one.
template <int S, int CHUNK, int BN>
__global__ void __launch_bounds__(OZ_THREADS, 1)
oz_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
               OzArgs a) {
  // a stopped iteration: every CTA leaves before any barrier or TMEM set-up
  if (skipped(a.skip)) return;
  constexpr int A_TILE = OZ_BM * OZ_ROW_BYTES;  // bytes per A-plane tile
  constexpr int B_TILE = BN * OZ_ROW_BYTES;  // bytes per B-plane tile
  constexpr int STAGE = S * (A_TILE + B_TILE);
  constexpr int NBUF = OZ_TMEM_COLS / (S * BN);  // accumulator buffers
  constexpr int EPI_COLS = BN * 4 / OZ_EPI_WARPS;  // output columns per epilogue thread
  static_assert(NBUF >= 1 && NBUF <= 2, "one or two TMEM accumulator sets of S groups");
  static_assert(S % 2 == 0 && S * CHUNK * OZ_BK * 64 * 64 <= (1 << 24),
                "exact group sums over a chunk");
  constexpr bool kSmallChunk = S * CHUNK * OZ_BK * 64 * 64 <= (1 << 22);
  extern __shared__ __align__(1024) unsigned char oz_smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)oz_smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full_bar[OZ_STAGES], empty_bar[OZ_STAGES];
  __shared__ __align__(8) uint64_t acc_full[NBUF], acc_empty[NBUF], drain_bar;
  __shared__ uint32_t tmem_base_s;
  __shared__ int abort_s;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nwork = a.tiles_m * a.tiles_n * a.splits;

  if (tid == 0) {
    abort_s = 0;
    for (int s = 0; s < OZ_STAGES; s++) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    for (int b = 0; b < NBUF; b++) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 32 * OZ_EPI_WARPS);
    }
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

  // Persistent loop: this CTA takes work items blockIdx.x, blockIdx.x +
  // gridDim.x, ...  Stage and barrier phases run on across items, so the TMA
  // warp streams the next item's planes while the MMAs of the current one
  // run, and the MMA warp starts the next item as soon as the epilogue has
  // drained the accumulators (before the epilogue's final FP64 assembly and
  // C update).
  if (warp == OZ_TMA_WARP) {
    // ------------------------------------------------------------ TMA producer
    if (lane == 0) {
      int it = 0;  // K-steps issued by this CTA
      bool live = true;
      for (int w = blockIdx.x; w < nwork && live; w += gridDim.x) {
        const OzWork o = oz_work(a, w, BN);
        for (int kt = 0; kt < o.nkt; kt++, it++) {
          const int s = it % OZ_STAGES;
          if (it >= OZ_STAGES &&
              !mbar_wait(&empty_bar[s], ((it / OZ_STAGES) - 1) & 1, abort_flag, a.status)) {
            live = false;
            break;
          }
          unsigned char* st = smem + s * STAGE;
          mbar_expect_tx(&full_bar[s], STAGE);
          const int kc = (o.kt0 + kt) * OZ_BK;
          tma_load_3d(st, &tmA, &full_bar[s], kc, o.m0, 0);
          tma_load_3d(st + S * A_TILE, &tmB, &full_bar[s], kc, o.n0, 0);
        }
      }
      // drain: every issued stage must have landed before the CTA can exit
      for (int k = (it > OZ_STAGES ? it - OZ_STAGES : 0); k < it; k++) {
        long long spins = 0;
        while (!mbar_try(&full_bar[k % OZ_STAGES], (k / OZ_STAGES) & 1) && ++spins < OZ_SPIN) {
        }
      }
    }
  } else if (warp == OZ_MMA_WARP) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      int it = 0, ch = 0;  // K-steps consumed, accumulator chunks completed
      bool live = true;
      for (int w = blockIdx.x; w < nwork && live; w += gridDim.x) {
        const OzWork o = oz_work(a, w, BN);
        for (int kt = 0; kt < o.nkt; kt++, it++) {
          const int s = it % OZ_STAGES;
          const bool chunk_first = (kt % CHUNK) == 0;
          // accumulator set of this chunk; its previous chunk must be drained
          const int buf = ch % NBUF;
          const uint32_t tacc = tmem + (uint32_t)(buf * S * BN);
          if (chunk_first && ch >= NBUF &&
              !mbar_wait(&acc_empty[buf], ((ch / NBUF) - 1) & 1, abort_flag, a.status)) {
            live = false;
            break;
          }
          if (!mbar_wait(&full_bar[s], (it / OZ_STAGES) & 1, abort_flag, a.status)) {
            live = false;
            break;
          }
          tc_fence_after();
          const uint32_t sa = smem_u32(smem + s * STAGE);
          const uint32_t sb = sa + S * A_TILE;
          // group d = p + q accumulates in TMEM columns (d - 2) * 64 .. +63;
          // the first MMA of a group in a chunk overwrites its accumulator
          if (a.merged) {
            // A plane p against the B planes q = 1 .. S + 1 - p at once: the
            // B plane tiles lie back to back in shared memory (one K-major
            // operand of 64 rows per plane) and their groups p + q are
            // adjacent TMEM column blocks, so up to four planes form one
            // MMA of N = 256 (12 MMAs per K step instead of 36, the A tile
            // read once per four B planes).  Plane 1's MMAs cover every
            // group and come first.
#pragma unroll
            for (int ks = 0; ks < OZ_BK / 16; ks++) {
#pragma unroll
              for (int p = 1; p <= S; p++) {
                const uint64_t ad = oz_desc(sa + (p - 1) * A_TILE + ks * 32);
#pragma unroll
                for (int q0 = 1; q0 <= S + 1 - p; q0 += 4) {
                  const int nq = (S + 2 - p - q0) < 4 ? (S + 2 - p - q0) : 4;
                  const uint64_t bd = oz_desc(sb + (q0 - 1) * B_TILE + ks * 32);
                  umma(tacc + (p + q0 - 2) * BN, ad, bd,
                       (chunk_first && p == 1 && ks == 0) ? 0u : 1u, oz_idesc(nq * BN));
                }
              }
            }
          } else {
#pragma unroll
            for (int d = 2; d <= S + 1; d++) {
#pragma unroll
              for (int p = 1; p < d; p++) {
                const int q = d - p;
#pragma unroll
                for (int ks = 0; ks < OZ_BK / 16; ks++) {
                  const uint64_t ad = oz_desc(sa + (p - 1) * A_TILE + ks * 32);
                  const uint64_t bd = oz_desc(sb + (q - 1) * B_TILE + ks * 32);
                  umma(tacc + (d - 2) * BN, ad, bd,
                       (chunk_first && p == 1 && ks == 0) ? 0u : 1u, oz_idesc(BN));
                }
              }
            }
          }
          umma_commit(&empty_bar[s]);
          const bool chunk_last = ((kt + 1) % CHUNK) == 0 || kt + 1 == o.nkt;
          if (chunk_last) {
            umma_commit(&acc_full[buf]);
            ch++;
          }
        }
      }
      // every MMA issued must have completed before TMEM is released
      umma_commit(&drain_bar);
      long long spins = 0;
      while (!mbar_try(&drain_bar, 0) && ++spins < OZ_SPIN) {
      }
    }
  } else {
    // ------------------------------------------------------------ epilogue warps 0-7
    // thread: output row r (TMEM lane), columns cb .. cb + EPI_COLS - 1
    constexpr int HG = S / 2;                  // groups d = 2 .. HG + 1 form the high part
    constexpr int LO_BITS = OZ_BITS * HG;      // low part: 2^-LO_BITS units of the high part
    constexpr int SH = 2 * OZ_BITS + OZ_BITS * (HG - 1) - 2 * OZ_HEADROOM;
    const int r = (warp & 3) * 32 + lane;
    const int cb = (warp >> 2) * EPI_COLS;
    const uint32_t lane_addr = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)cb;
    int ch = 0;
    bool ok = true;
    for (int w = blockIdx.x; w < nwork && ok; w += gridDim.x) {
      const OzWork o = oz_work(a, w, BN);
      const int nchunks = (o.nkt + CHUNK - 1) / CHUNK;
      double* const part = o.part;
      const bool beta0 = part != nullptr || a.beta == 0.0, beta1 = a.beta == 1.0;
      const int gi = o.m0 + r, n0 = o.n0;
      double* const Cp = a.C;
      const int64_t ldc = a.ldc;
      const int cpx = a.cpx, Nc = a.Nc;
      long long hi[EPI_COLS];  // units 2^(-OZ_BITS (HG - 1)) of the group-2 scale
      int lo[EPI_COLS];        // units 2^(-OZ_BITS (S - 1)), in [0, 2^LO_BITS)
#pragma unroll
      for (int c = 0; c < EPI_COLS; c++) {
        hi[c] = 0;
        lo[c] = 0;
      }
      for (int chunk = 0; chunk < nchunks; chunk++, ch++) {
        if (chunk == nchunks - 1 && !beta0 && gi < a.M) {
          // the C tile is read once, after the last chunk: pull it into L2
          // while the chunk's MMAs run
#pragma unroll 4
          for (int c = 0; c < EPI_COLS; c++) {
            const int gj = n0 + cb + c;
            if (gj < a.Nl) asm volatile("prefetch.global.L2 [%0];" ::"l"(oz_out_ptr(Cp, ldc, cpx, Nc, gi, gj)));
          }
        }
        const int buf = ch % NBUF;
        ok = mbar_wait_backoff(&acc_full[buf], (ch / NBUF) & 1, abort_flag, a.status);
        if (!ok) break;
        tc_fence_after();
        // 4 columns at a time: the register file is split over the four SM
        // sub-partitions, so with 10 warps a thread has at most 168 registers
#pragma unroll
        for (int c0 = 0; c0 < EPI_COLS; c0 += 4) {
          float sv[S][4];
#pragma unroll
          for (int g = 0; g < S; g++) tmem_ld4(lane_addr + (uint32_t)((buf * S + g) * BN + c0), sv[g]);
          tmem_wait_ld();
#pragma unroll
          for (int j = 0; j < 4; j++) {
            // group d = g + 2 holds an integer times 2^(-7g): scale by 2^(7g)
            // (exact) and convert exactly
            long long th = 0, tl = 0;
            if constexpr (kSmallChunk && S == 8) {
              // |k| <= 2^22: pairs k_a 2^7 + k_b stay below 2^30 in int32
              int k[S];
#pragma unroll
              for (int g = 0; g < S; g++) k[g] = group_int_small(sv[g][j], g);
              const int p01 = k[0] * (1 << OZ_BITS) + k[1], p23 = k[2] * (1 << OZ_BITS) + k[3];
              const int p45 = k[4] * (1 << OZ_BITS) + k[5], p67 = k[6] * (1 << OZ_BITS) + k[7];
              th = (long long)p01 * (1ll << (2 * OZ_BITS)) + p23;
              tl = (long long)p45 * (1ll << (2 * OZ_BITS)) + p67;
            } else {
#pragma unroll
              for (int g = 0; g < S; g++) {
                const long long v = group_int(sv[g][j], g);
                if (g < HG) th += v << (OZ_BITS * (HG - 1 - g));
                else tl += v << (OZ_BITS * (S - 1 - g));
              }
            }
            tl += lo[c0 + j];
            hi[c0 + j] += th + (tl >> LO_BITS);  // arithmetic shift: floor
            lo[c0 + j] = (int)(tl & ((1ll << LO_BITS) - 1));
          }
        }
        // accumulators drained: the MMA warp may overwrite them
        tc_fence_before();
        mbar_arrive(&acc_empty[buf]);
      }
      if (ok && gi < a.M) {
        // final: value = (hi 2^LO_BITS + lo) 2^(E_i + F_j - SH - LO_BITS) alpha,
        // one rounding to FP64 by integer operations.  One loop per (alpha,
        // beta) case, so that no FP64 work of the other cases is executed
        // speculatively; C is read in batches of 8 columns.
        const int e_row = exp_of_absbits(a.bitsA[gi]) - SH - LO_BITS;
        const double alpha = part ? 1.0 : a.alpha;
        const bool unit = alpha == 1.0 || alpha == -1.0;
        const bool flip = alpha == -1.0;
        const int mode = part ? 0 : (!unit ? 3 : (beta0 ? 0 : (beta1 ? 1 : 2)));
        if (mode == 0) {
#pragma unroll
          for (int c = 0; c < EPI_COLS; c++) {
            const int gj = n0 + cb + c;
            if (gj >= a.Nl) continue;
            const double v = fx_to_double(hi[c], (unsigned)lo[c], LO_BITS, e_row + exp_of_absbits(a.bitsB[gj]), flip);
            if (part) part[(int64_t)gj * a.M + gi] = v;  // split-K partial, ld = M
            else *oz_out_ptr(Cp, ldc, cpx, Nc, gi, gj) = v;
          }
        } else {
#pragma unroll
          for (int c0 = 0; c0 < EPI_COLS; c0 += 8) {
            double cv[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
              const int gj = n0 + cb + c0 + j;
              cv[j] = gj < a.Nl ? *oz_out_ptr(Cp, ldc, cpx, Nc, gi, gj) : 0.0;
            }
#pragma unroll
            for (int j = 0; j < 8; j++) {
              const int c = c0 + j, gj = n0 + cb + c;
              if (gj >= a.Nl) continue;
              double v = fx_to_double(hi[c], (unsigned)lo[c], LO_BITS, e_row + exp_of_absbits(a.bitsB[gj]), flip);
              if (mode == 1) v = cv[j] + v;
              else if (mode == 2) v = fma(a.beta, cv[j], v);
              else v = fma(alpha, v, beta0 ? 0.0 : a.beta * cv[j]);
              *oz_out_ptr(Cp, ldc, cpx, Nc, gi, gj) = v;
            }
          }
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
                                 double beta, const int* skip) {
  if (skipped(skip)) return;
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

// A real operand without a structure mask is read through its pointer
// directly: element (r, k) of the logical operand sits at r + k ld when the
// operand is contiguous along r, else at k + r ld (transposition is the
// identity on real data).  Other operands go through oz_fetch.
template <class T>
__device__ __forceinline__ bool oz_plain(const OzSrc<T>& s) {
  return !traits<T>::cpx && s.op.mask == MASK_FULL;
}


// Row maxima of |X| as IEEE bit patterns (non-negative doubles order like
// their bits), accumulated with atomicMax over a 2-D grid of (rows, K
// chunks) so that tall K ranges are read by many CTAs in parallel.
constexpr int OZ_EXP_KCHUNK = 1024;
template <class T>
__global__ void __launch_bounds__(256) oz_absmax_kernel(OzSrc<T> sa, int Ra,
                                                        unsigned long long* bits_a, OzSrc<T> sb,
                                                        int Rb, unsigned long long* bits_b, int K,
                                                        const int* skip) {
  if (skipped(skip)) return;
  // blockIdx.z: 0 the rows of op(A), 1 the columns of op(B)
  const OzSrc<T>& s = blockIdx.z == 0 ? sa : sb;
  const int R = blockIdx.z == 0 ? Ra : Rb;
  unsigned long long* mx_bits = blockIdx.z == 0 ? bits_a : bits_b;
  const int k0 = blockIdx.y * OZ_EXP_KCHUNK;
  const int k1 = min(K, k0 + OZ_EXP_KCHUNK);
  if (oz_contig_r(s)) {
    // 256 consecutive rows per CTA, each thread walks the chunk of K
    const int r = blockIdx.x * 256 + threadIdx.x;
    if (r >= R) return;
    unsigned long long mx = 0;
    int k = k0;
    if (oz_plain(s)) {
      // eight independent loads in flight per thread
      const double* q = reinterpret_cast<const double*>(s.op.p) + r;
      const int64_t ld = s.op.ld;
      for (; k + 7 < k1; k += 8) {
        unsigned long long b[8];
#pragma unroll
        for (int i = 0; i < 8; i++) b[i] = absbits(q[(int64_t)(k + i) * ld]);
#pragma unroll
        for (int i = 0; i < 8; i++) mx = b[i] > mx ? b[i] : mx;
      }
    }
    for (; k < k1; k++) {
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
    int k = k0 + lane;
    if (oz_plain(s)) {
      const double* q = reinterpret_cast<const double*>(s.op.p) + (int64_t)r * s.op.ld;
      for (; k + 7 * 32 < k1; k += 8 * 32) {
        unsigned long long b[8];
#pragma unroll
        for (int i = 0; i < 8; i++) b[i] = absbits(q[k + 32 * i]);
#pragma unroll
        for (int i = 0; i < 8; i++) mx = b[i] > mx ? b[i] : mx;
      }
    }
    for (; k < k1; k += 32) {
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
// Row maxima of both operands in one launch into bits_a[0, Ra) and
// bits_b[0, Rb); the nbits words from bits_a on (which hold both) are
// zeroed first
template <class T>
static int oz_exponents(cudaStream_t st, const OzSrc<T>& sa, int Ra, unsigned long long* bits_a,
                        const OzSrc<T>& sb, int Rb, unsigned long long* bits_b, int K,
                        int64_t nbits) {
  MAK_CUDA_TRY(cudaMemsetAsync(bits_a, 0, (size_t)nbits * sizeof(unsigned long long), st));
  const unsigned gy = (unsigned)ceil_div(K > 0 ? K : 1, OZ_EXP_KCHUNK);
  const int64_t gxa = oz_contig_r(sa) ? ceil_div(Ra, 256) : ceil_div(Ra, 8);
  const int64_t gxb = oz_contig_r(sb) ? ceil_div(Rb, 256) : ceil_div(Rb, 8);
  const unsigned gx = (unsigned)(gxa > gxb ? gxa : gxb);
  note_launch();
  oz_absmax_kernel<T><<<dim3(gx, gy, 2), 256, 0, st>>>(sa, Ra, bits_a, sb, Rb, bits_b, K,
                                                        skip_flag());
  return cudaGetLastError() == cudaSuccess ? 0 : MAK_ERR_CUDA;
}

// planes[p][r][k] (Rpad x Kpad, bf16) = sign * digit_p * 2^(-7(p-1)), zero padded
// (blockIdx.z: 0 the rows of op(A), 1 the columns of op(B); one launch)
struct OzPlaneOut {
  int R, Rpad;
  const unsigned long long* bits;  // largest magnitude of each row, IEEE bits
  __nv_bfloat16* planes;
};
template <class T, int S>
__global__ void __launch_bounds__(256) oz_split_kernel(OzSrc<T> sa, OzPlaneOut oa, OzSrc<T> sb,
                                                       OzPlaneOut ob, int K, int Kpad,
                                                       const int* skip) {
  if (skipped(skip)) return;
  const OzSrc<T>& s = blockIdx.z == 0 ? sa : sb;
  const OzPlaneOut& o = blockIdx.z == 0 ? oa : ob;
  const int R = o.R, Rpad = o.Rpad;
  __nv_bfloat16* planes = o.planes;
  const int r0 = blockIdx.y * 64, k0 = blockIdx.x * 64;
  if (r0 >= Rpad) return;  // the shorter side's grid rows (uniform per CTA)
  // row stride 68 doubles: the digit phase's reads (eight rows of eight
  // threads, eight apart in k) fall on distinct banks pairwise
  __shared__ double tile[64][68];
  // bf16 bits of +-(t - 64) 2^(-7p) for the biased digits t = 0 .. 128 of
  // plane p ([0]: positive values, [1]: negated)
  __shared__ unsigned short lut[2][S][130];
  const int tid = threadIdx.x;
  const bool cr = oz_contig_r(s);
  for (int e = tid; e < 2 * S * 129; e += 256) {
    const int sg = e / (S * 129), p = (e / 129) % S, t = e % 129;
    const float v = ldexpf((float)(t - 64), -OZ_BITS * p);
    lut[sg][p][t] = __bfloat16_as_ushort(__float2bfloat16_rn(sg && t != 64 ? -v : v));
  }
  if (oz_plain(s)) {
    // sixteen independent loads per thread, then the stores to the tile
    const double* src = reinterpret_cast<const double*>(s.op.p);
    const int64_t ld = s.op.ld;
    double v[16];
#pragma unroll
    for (int i = 0; i < 16; i++) {
      const int e = tid + 256 * i;
      int rr, kk;
      if (cr) { rr = e % 64; kk = e / 64; } else { kk = e % 64; rr = e / 64; }
      const int r = r0 + rr, k = k0 + kk;
      v[i] = (r < R && k < K) ? src[cr ? (int64_t)r + (int64_t)k * ld : (int64_t)k + (int64_t)r * ld]
                              : 0.0;
    }
#pragma unroll
    for (int i = 0; i < 16; i++) {
      const int e = tid + 256 * i;
      int rr, kk;
      if (cr) { rr = e % 64; kk = e / 64; } else { kk = e % 64; rr = e / 64; }
      tile[rr][kk] = v[i];
    }
  } else {
    for (int e = tid; e < 64 * 64; e += 256) {
      int rr, kk;
      if (cr) { rr = e % 64; kk = e / 64; } else { kk = e % 64; rr = e / 64; }
      const int r = r0 + rr, k = k0 + kk;
      tile[rr][kk] = (r < R && k < K) ? oz_fetch(s, r, k) : 0.0;
    }
  }
  __syncthreads();
  constexpr int FB = OZ_BITS * S;  // fractional bits of the fixed-point value
  static_assert(FB <= 56, "the fixed-point value fits 28 + 28 bits");
  const size_t plane_stride = (size_t)Rpad * Kpad;
  // each thread: one row, eight adjacent k (one 16-byte store per plane).
  // Digits are cut with 32-bit integer operations (the value as two 28-bit
  // halves) and each bf16 plane value d 2^(-7p) is assembled from a table of
  // the bf16 bit patterns of the digits -64..64 by lowering the exponent
  // field by 7p: no conversion instructions.
  for (int e = tid; e < 64 * 8; e += 256) {
    const int rr = e / 8, kq = (e % 8) * 8;
    const int r = r0 + rr;
    const int k = k0 + kq;
    if (r >= Rpad || k >= Kpad) continue;
    const int Fr = ((r < R) ? exp_of_absbits(o.bits[r]) : 0) + OZ_HEADROOM;  // frame: |x| < 2^(Fr - 1)
    unsigned packed[S][4];
#pragma unroll
    for (int h = 0; h < 8; h++) {
      const double x = tile[rr][kq + h];
      const unsigned long long bts = (unsigned long long)__double_as_longlong(x);
      const bool neg = (bts >> 63) != 0;
      int ex = (int)((bts >> 52) & 0x7FF);
      unsigned long long m = bts & 0x000FFFFFFFFFFFFFull;
      if (ex == 0) ex = 1; else m |= 0x0010000000000000ull;
      // f = |x| 2^(FB - Fr) rounded to nearest: f <= 2^(FB - 1)
      const int sh = ex - 1075 + FB - Fr;
      unsigned long long f;
      if ((bts & 0x7FFFFFFFFFFFFFFFull) == 0) f = 0;
      else if (sh >= 0) f = (sh >= 11) ? 0 : (m << sh);
      else if (-sh >= 55) f = 0;
      else f = (m >> (-sh)) + ((m >> (-sh - 1)) & 1ull);
      // balanced base-2^7 digits d_p (plane p weighs 2^(-7p)): d_p in
      // [-64, 63] below the leading digit, which is in [0, 64].  Adding
      // 64 to every digit position (the constant BIAS) turns the balanced
      // digits into the plain base-128 digits t_p = d_p + 64 of f + BIAS, so
      // each is one shift and one mask, with no carries
      constexpr unsigned long long BIAS = [] {
        unsigned long long b = 0;
        for (int i = 0; i < S; i++) b |= 64ull << (OZ_BITS * i);
        return b;
      }();
      const unsigned long long u = f + BIAS;
      const unsigned short* tb = &lut[neg ? 1 : 0][0][0];
#pragma unroll
      for (int p = 0; p < S; p++) {
        unsigned t = (unsigned)(u >> (OZ_BITS * (S - 1 - p)));
        // the leading digit is at most 64 when |x| < 2^(Fr - 1); the bound
        // also keeps the table index in range for an operand that changed
        // between the two passes
        t = p == 0 ? (t < 128u ? t : 128u) : (t & 127u);
        const unsigned b = tb[p * 130 + t];
        if (h & 1) packed[p][h >> 1] |= b << 16;
        else packed[p][h >> 1] = b;
      }
    }
#pragma unroll
    for (int p = 0; p < S; p++)
      *reinterpret_cast<uint4*>(planes + p * plane_stride + (size_t)r * Kpad + k) =
          make_uint4(packed[p][0], packed[p][1], packed[p][2], packed[p][3]);
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
  // one box holds all S planes of a K step (plane p at p * box_rows rows),
  // so a stage takes two copies instead of 2 S
  cuuint32_t box[3] = {(cuuint32_t)OZ_BK, (cuuint32_t)box_rows, (cuuint32_t)S};
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE,
                  OZ_ROW_BYTES == 32 ? CU_TENSOR_MAP_SWIZZLE_32B
                                     : (OZ_ROW_BYTES == 64 ? CU_TENSOR_MAP_SWIZZLE_64B
                                                           : CU_TENSOR_MAP_SWIZZLE_128B),
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : MAK_ERR_CUDA;
}

template <int S, int BN>
static size_t oz_smem_bytes() {
  return (size_t)OZ_STAGES * S * (OZ_BM * OZ_BK * 2 + BN * OZ_BK * 2) + 1024;
}

// the kernels' dynamic shared-memory limit, raised once per device
template <int S>
static void oz_set_attr() {
  static PerDevice<int> pd;
  pd.get([] {
    cudaFuncSetAttribute(oz_gemm_kernel<S, OZ_KSTEPS_PER_CHUNK, 64>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)oz_smem_bytes<S, 64>());
    cudaFuncSetAttribute(oz_gemm_kernel<S, OZ_SMALL_CHUNK, 64>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)oz_smem_bytes<S, 64>());
    cudaFuncSetAttribute(oz_gemm_kernel<S, OZ_SMALL_CHUNK, 32>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)oz_smem_bytes<S, 32>());
    return 1;
  });
}

// slices: 8 (56-bit fixed point) for Float64 data, 4 (28-bit) for Float32 data
template <class T>
constexpr int oz_slices() { return sizeof(real_t<T>) == 8 ? 8 : 4; }

template <class T>
int oz_gemm(cudaStream_t st, int64_t M, int64_t N, int64_t K, T alpha, Operand<T> A, Operand<T> B,
            T beta, T* C, int64_t ldc, Arena& ar, int* status, int max_ctas) {
  constexpr bool cpx = traits<T>::cpx;
  constexpr int S = oz_slices<T>();
  const int64_t Kl = cpx ? 2 * K : K;       // logical K
  const int64_t Nl = cpx ? 2 * N : N;       // logical output columns
  const int64_t Mpad = ceil_div(M > 0 ? M : 1, OZ_BM) * OZ_BM;
  const int64_t Kpad = ceil_div(Kl > 0 ? Kl : 1, OZ_BK) * OZ_BK;
  const int64_t nkt_total = Kpad / OZ_BK;
  // products with K <= 128 (one short chunk per tile) take 32-wide tiles with
  // two accumulator sets, so that a tile's MMAs overlap the previous tile's
  // epilogue; longer products the 64-wide tile (MAK_OZ_NARROW = 0: always 64)
  const bool small = nkt_total * OZ_BK <= 128;
  const int BN = (small && tuning(TUNE_OZ_NARROW) != 0) ? 32 : 64;
  const int64_t Npad = ceil_div(Nl > 0 ? Nl : 1, (int64_t)BN) * BN;
  const int64_t Npad64 = ceil_div(Nl > 0 ? Nl : 1, (int64_t)64) * 64;  // workspace bound
  const int64_t tiles = (Mpad / OZ_BM) * (Npad / BN);
  // persistent grid cap: the caller's limit, else the thread's budget, else every SM
  if (max_ctas <= 0) max_ctas = split_gemm_cta_budget();
  const int cap = (max_ctas > 0 && max_ctas < num_sms()) ? max_ctas : num_sms();
  // split K (whole chunks per split) when the tiles alone leave CTAs idle:
  // the count minimising waves x (chunks per item + the item's fixed cost,
  // about half a chunk of epilogue), with at most two waves of items so the
  // partials stay within the measured bound.  A ragged last wave idles the
  // grid (64 tiles x 3 splits on 152 CTAs: 2 waves at 63 %), so the count is
  // chosen by the waves it takes, not by the CTAs it would fill.
  int splits = 1;
  {
    const int64_t nchunk = ceil_div(nkt_total, OZ_KSTEPS_PER_CHUNK);
    if (tiles < cap && nchunk > 1) {
      double best = 0.0;
      for (int s = 1; s <= 32 && s <= nchunk; s++) {
        const int64_t cps = ceil_div(nchunk, (int64_t)s);
        const int64_t s_eff = ceil_div(nchunk, cps);
        const int64_t items = tiles * s_eff;
        if (s > 1 && items > 2 * (int64_t)cap) break;
        const double cost = (double)ceil_div(items, (int64_t)cap) * ((double)cps + 0.5);
        if (s == 1 || cost < best * 0.999) {
          best = cost;
          splits = (int)s_eff;
        }
      }
    }
  }
  const int64_t chunks_per_split =
      ceil_div(ceil_div(nkt_total, OZ_KSTEPS_PER_CHUNK), splits);
  splits = (int)ceil_div(ceil_div(nkt_total, OZ_KSTEPS_PER_CHUNK), chunks_per_split);

  unsigned long long* bitsA = ar.take<unsigned long long>(Mpad + Npad64);
  unsigned long long* bitsB = bitsA + Mpad;
  __nv_bfloat16* PA = ar.take<__nv_bfloat16>((size_t)S * Mpad * Kpad);
  __nv_bfloat16* PB = ar.take<__nv_bfloat16>((size_t)S * Npad64 * Kpad);
  // split-K partials; a measuring pass reserves a bound that holds for every
  // smaller output as well (splitting happens only when tiles < SMs, and then
  // splits * tiles < 2 * SMs), because call sites measure at their largest
  // shape while the split count grows as the output shrinks
  double* part = nullptr;
  if (ar.base == nullptr) {
    if (nkt_total > OZ_KSTEPS_PER_CHUNK) {
      const size_t bound = (size_t)2 * num_sms() * OZ_BM * OZ_BN;
      const size_t cap32 = (size_t)32 * Mpad * Npad;
      ar.take<double>(bound < cap32 ? bound : cap32);
    }
  } else if (splits > 1) {
    part = ar.take<double>((size_t)splits * M * Nl);
  }
  if (ar.base == nullptr) return 0;
  if (!ar.ok()) return MAK_ERR_WORKSPACE;
  if (M <= 0 || N <= 0) return 0;

  OzSrc<T> sa{A, 0, (int)M, (int)K};
  OzSrc<T> sb{B, 1, (int)N, (int)K};
  MAK_TRY(oz_exponents<T>(st, sa, (int)M, bitsA, sb, (int)Nl, bitsB, (int)Kl, Mpad + Npad));
  {
    const OzPlaneOut oa{(int)M, (int)Mpad, bitsA, PA}, ob{(int)Nl, (int)Npad, bitsB, PB};
    const int64_t rows = Mpad > Npad ? Mpad : Npad;
    note_launch();
    oz_split_kernel<T, S><<<dim3((unsigned)ceil_div(Kpad, 64), (unsigned)ceil_div(rows, 64), 2), 256, 0,
                            st>>>(sa, oa, sb, ob, (int)Kl, (int)Kpad, skip_flag());
    MAK_CUDA_TRY(cudaGetLastError());
  }

  CUtensorMap mapA, mapB;
  MAK_TRY(make_plane_map(&mapA, PA, S, (int)Mpad, (int)Kpad, OZ_BM));
  MAK_TRY(make_plane_map(&mapB, PB, S, (int)Npad, (int)Kpad, BN));
  oz_set_attr<S>();

  const double ar_ = re_(alpha), br_ = re_(beta);
  const double work = (cpx ? 8.0 : 2.0) * (double)M * N * K;
  ProfScope prof(st, PROF_GEMM_MIXED, work);
  {
    // persistent grid: one CTA per SM (shared memory holds one CTA), each
    // looping over work items
    const int split_steps = (int)(chunks_per_split * OZ_KSTEPS_PER_CHUNK);
    const int tm = (int)(Mpad / OZ_BM), tn = (int)(Npad / BN);
    OzArgs args{(int)M, (int)Nl, (int)nkt_total, split_steps, tm, tn, splits, bitsA, bitsB,
                (double*)C, ldc, cpx ? 1 : 0, (int)N, ar_, br_, part, part ? M * Nl : 0,
                status, skip_flag(), tuning(TUNE_OZ_MERGED) != 0 ? 1 : 0};
    const int64_t nwork = (int64_t)tm * tn * splits;
    const int grid = (int)(nwork < cap ? nwork : cap);
    note_launch();
    if (small && BN == 32)  // one short chunk: the FFMA conversion
      oz_gemm_kernel<S, OZ_SMALL_CHUNK, 32>
          <<<grid, OZ_THREADS, oz_smem_bytes<S, 32>(), st>>>(mapA, mapB, args);
    else if (small)
      oz_gemm_kernel<S, OZ_SMALL_CHUNK, 64>
          <<<grid, OZ_THREADS, oz_smem_bytes<S, 64>(), st>>>(mapA, mapB, args);
    else
      oz_gemm_kernel<S, OZ_KSTEPS_PER_CHUNK, 64>
          <<<grid, OZ_THREADS, oz_smem_bytes<S, 64>(), st>>>(mapA, mapB, args);
    MAK_CUDA_TRY(cudaGetLastError());
  }
  if (part) {
    note_launch();
    oz_reduce_kernel<<<(unsigned)ceil_div(M * Nl, 256), 256, 0, st>>>(
        (int)M, (int)Nl, splits, part, M * Nl, (double*)C, ldc, cpx ? 1 : 0, (int)N, ar_, br_,
        skip_flag());
    MAK_CUDA_TRY(cudaGetLastError());
  }
  return 0;
}

#define MAK_INST_OZ(T)                                                                        \
  template int oz_gemm<T>(cudaStream_t, int64_t, int64_t, int64_t, T, Operand<T>, Operand<T>, \
                          T, T*, int64_t, Arena&, int*, int);
MAK_INST_OZ(double)
MAK_INST_OZ(zcomplex)

}  // namespace mak
