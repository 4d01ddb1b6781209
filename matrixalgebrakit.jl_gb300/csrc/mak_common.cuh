// Shared device/host helpers for the GB300 orthogonal-factorization library.
//
// Scalar model: the four LAPACK element types Float64 (d), ComplexF64 (z),
// Float32 (s), ComplexF32 (c); complex values are stored interleaved
// (re, im) exactly like Julia's ComplexF64/ComplexF32 and C99 complex, so a
// CuMatrix{ComplexF64} pointer can be passed straight through the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#include <atomic>
#include <mutex>

#include "../../include/mak_gb300.h"

namespace mak {

// ------------------------------------------------------------ complex type --
template <class R>
struct __align__(2 * sizeof(R)) cplx {
  R re, im;
  __host__ __device__ cplx() {}
  __host__ __device__ constexpr cplx(R r) : re(r), im(0) {}
  __host__ __device__ constexpr cplx(R r, R i) : re(r), im(i) {}
};
template <class R> __host__ __device__ __forceinline__ cplx<R> operator+(cplx<R> a, cplx<R> b) { return {a.re + b.re, a.im + b.im}; }
template <class R> __host__ __device__ __forceinline__ cplx<R> operator-(cplx<R> a, cplx<R> b) { return {a.re - b.re, a.im - b.im}; }
template <class R> __host__ __device__ __forceinline__ cplx<R> operator-(cplx<R> a) { return {-a.re, -a.im}; }
template <class R> __host__ __device__ __forceinline__ cplx<R> operator*(cplx<R> a, cplx<R> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <class R> __host__ __device__ __forceinline__ cplx<R> operator*(R s, cplx<R> a) { return {s * a.re, s * a.im}; }
template <class R> __host__ __device__ __forceinline__ cplx<R> operator*(cplx<R> a, R s) { return {s * a.re, s * a.im}; }
template <class R> __host__ __device__ __forceinline__ cplx<R>& operator+=(cplx<R>& a, cplx<R> b) { a.re += b.re; a.im += b.im; return a; }
template <class R> __host__ __device__ __forceinline__ cplx<R>& operator-=(cplx<R>& a, cplx<R> b) { a.re -= b.re; a.im -= b.im; return a; }
template <class R> __host__ __device__ __forceinline__ bool operator==(cplx<R> a, cplx<R> b) { return a.re == b.re && a.im == b.im; }

using zcomplex = cplx<double>;
using ccomplex = cplx<float>;

// ------------------------------------------------------------ scalar traits --
template <class T> struct traits;
template <> struct traits<double> { using real = double; static constexpr bool cpx = false; static constexpr int code = MAK_F64; };
template <> struct traits<float>  { using real = float;  static constexpr bool cpx = false; static constexpr int code = MAK_F32; };
template <> struct traits<zcomplex> { using real = double; static constexpr bool cpx = true; static constexpr int code = MAK_C64; };
template <> struct traits<ccomplex> { using real = float;  static constexpr bool cpx = true; static constexpr int code = MAK_C32; };
template <class T> using real_t = typename traits<T>::real;

__host__ __device__ __forceinline__ double conj_(double x) { return x; }
__host__ __device__ __forceinline__ float conj_(float x) { return x; }
template <class R> __host__ __device__ __forceinline__ cplx<R> conj_(cplx<R> x) { return {x.re, -x.im}; }

__host__ __device__ __forceinline__ double re_(double x) { return x; }
__host__ __device__ __forceinline__ float re_(float x) { return x; }
template <class R> __host__ __device__ __forceinline__ R re_(cplx<R> x) { return x.re; }
__host__ __device__ __forceinline__ double im_(double) { return 0.0; }
__host__ __device__ __forceinline__ float im_(float) { return 0.0f; }
template <class R> __host__ __device__ __forceinline__ R im_(cplx<R> x) { return x.im; }

__host__ __device__ __forceinline__ double abs2_(double x) { return x * x; }
__host__ __device__ __forceinline__ float abs2_(float x) { return x * x; }
template <class R> __host__ __device__ __forceinline__ R abs2_(cplx<R> x) { return x.re * x.re + x.im * x.im; }

__host__ __device__ __forceinline__ double abs_(double x) { return fabs(x); }
__host__ __device__ __forceinline__ float abs_(float x) { return fabsf(x); }
__host__ __device__ __forceinline__ double abs_(cplx<double> x) { return hypot(x.re, x.im); }
__host__ __device__ __forceinline__ float abs_(cplx<float> x) { return hypotf(x.re, x.im); }

// fused multiply-add  acc + a*b
__device__ __forceinline__ double fma_(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fma_(float a, float b, float c) { return fmaf(a, b, c); }
template <class R> __device__ __forceinline__ cplx<R> fma_(cplx<R> a, cplx<R> b, cplx<R> c) {
  cplx<R> r;
  r.re = fma_(a.re, b.re, fma_(-a.im, b.im, c.re));
  r.im = fma_(a.re, b.im, fma_(a.im, b.re, c.im));
  return r;
}

template <class T> __host__ __device__ __forceinline__ T make_scalar(real_t<T> re, real_t<T> im);
template <> __host__ __device__ __forceinline__ double make_scalar<double>(double re, double) { return re; }
template <> __host__ __device__ __forceinline__ float make_scalar<float>(float re, float) { return re; }
template <> __host__ __device__ __forceinline__ zcomplex make_scalar<zcomplex>(double re, double im) { return {re, im}; }
template <> __host__ __device__ __forceinline__ ccomplex make_scalar<ccomplex>(float re, float im) { return {re, im}; }

template <class T> __host__ __device__ __forceinline__ T zero_() { return make_scalar<T>(0, 0); }
template <class T> __host__ __device__ __forceinline__ T one_() { return make_scalar<T>(1, 0); }

// multiplicative inverse of a scalar (complex: Smith-free plain formula with
// a single real division, adequate for the non-tiny values it is used on)
__device__ __forceinline__ double inv_(double x) { return 1.0 / x; }
__device__ __forceinline__ float inv_(float x) { return 1.0f / x; }
template <class R> __device__ __forceinline__ cplx<R> inv_(cplx<R> x) {
  R s = fabs(x.re) > fabs(x.im) ? fabs(x.re) : fabs(x.im);
  if (s == R(0)) return {R(1) / s, R(0)};
  R xr = x.re / s, xi = x.im / s;
  R d = (xr * xr + xi * xi) * s;
  return {xr / d, -xi / d};
}

// sign_safe (reference src/common/safemethods.jl:10-11):
// real: s < 0 ? -1 : +1 ; complex: s/|s| with 0 -> 1
__device__ __forceinline__ double sign_safe_(double s) { return s < 0.0 ? -1.0 : 1.0; }
__device__ __forceinline__ float sign_safe_(float s) { return s < 0.0f ? -1.0f : 1.0f; }
template <class R> __device__ __forceinline__ cplx<R> sign_safe_(cplx<R> s) {
  if (s.re == R(0) && s.im == R(0)) return {R(1), R(0)};
  R a = abs_(s);
  return {s.re / a, s.im / a};
}

// Reciprocal and square root for the panels' scalars.  GB300 issues about
// 1.6 FP64 operations per clock per SM, so a single thread's chain of
// dependent FP64 operations advances slowly, and IEEE division / square root
// sequences sit on every panel column's critical path.  Here both use the
// Newton-Raphson iteration (quadratic convergence; e.g. J.-M. Muller et
// al., Handbook of Floating-Point Arithmetic, ch. 5), seeded in single
// precision: 1/x by y <- y + y (1 - x y), 1/sqrt(x) by y <- y (3 - x y^2) / 2,
// then sqrt(x) = x y with one correction s <- s + (x - s^2) y / 2.  The
// argument is first reduced to [1, 2) (reciprocal) or [1, 4) (square root)
// by integer exponent arithmetic; |exponent| <= 1000 is required.
__device__ __forceinline__ double rcp_nr(double x) {
  const long long bits = __double_as_longlong(x);
  const int e = (int)((bits >> 52) & 0x7FF) - 1023;
  const double m = __longlong_as_double((bits & (long long)0x800FFFFFFFFFFFFFull) |
                                        0x3FF0000000000000ll);
  double y = (double)__frcp_rn((float)m);
  double r = fma(-m, y, 1.0);
  y = fma(y, r, y);
  r = fma(-m, y, 1.0);
  y = fma(y, r, y);
  return __longlong_as_double(__double_as_longlong(y) - ((long long)e << 52));
}
__device__ __forceinline__ double sqrt_nr(double x) {
  const long long bits = __double_as_longlong(x);
  const int e = (int)((bits >> 52) & 0x7FF) - 1023;
  const int k = e >> 1;  // floor(e / 2): x 2^-2k in [1, 4)
  const double m = __longlong_as_double(bits - ((long long)(2 * k) << 52));
  double y = (double)rsqrtf((float)m);
  y = y * fma(-0.5 * m * y, y, 1.5);
  y = y * fma(-0.5 * m * y, y, 1.5);
  double s = m * y;
  s = fma(fma(-s, s, m), 0.5 * y, s);
  return __longlong_as_double(__double_as_longlong(s) + ((long long)k << 52));
}
__device__ __forceinline__ float rcp_nr(float x) { return 1.0f / x; }
// sqrt of a non-negative sum of squares: the Newton form inside the normal
// range, the IEEE square root for 0, subnormals, huge values, Inf and NaN
__device__ __forceinline__ double sqrt_nr_safe(double x) {
  const int e = (int)((__double_as_longlong(x) >> 52) & 0x7FF) - 1023;
  return (x > 0.0 && e > -1000 && e < 1000) ? sqrt_nr(x) : sqrt(x);
}
__device__ __forceinline__ float sqrt_nr_safe(float x) { return sqrtf(x); }
__device__ __forceinline__ float sqrt_nr(float x) { return sqrtf(x); }
// exponent e of a positive finite x (x = f 2^e, f in [1, 2)); subnormals give -1023
__device__ __forceinline__ int exp2_of(double x) {
  return (int)((__double_as_longlong(x) >> 52) & 0x7FF) - 1023;
}
__device__ __forceinline__ int exp2_of(float x) { return (int)((__float_as_uint(x) >> 23) & 0xFF) - 127; }
__device__ __forceinline__ double pow2_(double, int e) { return __longlong_as_double((long long)(e + 1023) << 52); }
__device__ __forceinline__ float pow2_(float, int e) { return __uint_as_float((unsigned)(e + 127) << 23); }

// 1/x for the pivots and reflectors: the Newton form inside the normal
// range, IEEE division outside it (0, subnormals, huge values, Inf, NaN)
__device__ __forceinline__ double rcp_nr_safe(double x) {
  const int e = (int)((__double_as_longlong(x) >> 52) & 0x7FF) - 1023;
  return (e > -1000 && e < 1000) ? rcp_nr(x) : 1.0 / x;
}
__device__ __forceinline__ float rcp_nr_safe(float x) { return 1.0f / x; }
// 1/z for real and complex scalars (complex: conj(z) / |z|^2 with the
// components scaled by a power of two near |z|)
__device__ __forceinline__ double inv_fast(double x) { return rcp_nr_safe(x); }
__device__ __forceinline__ float inv_fast(float x) { return 1.0f / x; }
template <class R> __device__ __forceinline__ cplx<R> inv_fast(cplx<R> z) {
  const R w = fmax(fabs(z.re), fabs(z.im));
  if (!(w > R(0)) || !(w < R(INFINITY))) return inv_(z);
  const int e = exp2_of(w);
  const int lim = sizeof(R) == 8 ? 1000 : 100;
  if (e < -lim || e > lim) return inv_(z);
  const R sd = pow2_(R(0), -e);
  const R z1 = z.re * sd, z2 = z.im * sd;
  const R d = rcp_nr(fma_(z1, z1, z2 * z2)) * sd;
  return {z1 * d, -z2 * d};
}

// L1-bypassing loads for values written by other CTAs of the same launch
// (after a grid barrier); L1 is not coherent across SMs.
__device__ __forceinline__ double ld_cg(const double* p) { return __ldcg(p); }
__device__ __forceinline__ float ld_cg(const float* p) { return __ldcg(p); }
__device__ __forceinline__ zcomplex ld_cg(const zcomplex* p) {
  double2 v = __ldcg((const double2*)p);
  return {v.x, v.y};
}
__device__ __forceinline__ ccomplex ld_cg(const ccomplex* p) {
  float2 v = __ldcg((const float2*)p);
  return {v.x, v.y};
}
__device__ __forceinline__ int ld_cg(const int* p) { return __ldcg(p); }

// ------------------------------------------------------------ warp helpers --
__device__ __forceinline__ double shfl_xor_(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ float shfl_xor_(float v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
template <class R> __device__ __forceinline__ cplx<R> shfl_xor_(cplx<R> v, int m) {
  return {shfl_xor_(v.re, m), shfl_xor_(v.im, m)};
}
__device__ __forceinline__ double shfl_idx_(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ float shfl_idx_(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }
template <class R> __device__ __forceinline__ cplx<R> shfl_idx_(cplx<R> v, int src) {
  return {shfl_idx_(v.re, src), shfl_idx_(v.im, src)};
}
template <class T> __device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) v += shfl_xor_(v, m);
  return v;
}
template <class R> __device__ __forceinline__ R warp_max(R v) {
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) { R o = shfl_xor_(v, m); v = o > v ? o : v; }
  return v;
}

// Block-wide reductions (deterministic: fixed shuffle tree, fixed warp order).
// `sh` must hold 32 elements; every thread receives the result.
template <class T>
__device__ __forceinline__ T block_sum(T v, T* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  T r = zero_<T>();
  for (int w = 0; w < nw; w++) r += sh[w];
  return r;
}
template <class R>
__device__ __forceinline__ R block_max(R v, R* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_max(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  R r = sh[0];
  for (int w = 1; w < nw; w++) r = sh[w] > r ? sh[w] : r;
  return r;
}

// ------------------------------------------------------ bounded grid barrier --
// Used only inside cooperative launches (all CTAs are guaranteed co-resident).
// Every wait is bounded: after kSpinLimit polls the CTA records
// MAK_ERR_TIMEOUT in *status and the barrier reports failure, so a kernel can
// never hang the GPU.  `bar[0]` counts arrivals, `bar[1]` is the generation.
constexpr long long kSpinLimit = 1ll << 22;  // x >=64 ns sleep -> well under a minute

__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned nblocks, int* status,
                                             long long spin_limit = kSpinLimit) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    if (nblocks > 1) {
      volatile unsigned* vgen = bar + 1;
      unsigned g = *vgen;
      __threadfence();
      unsigned arrived = atomicAdd(bar, 1u);
      if (arrived == nblocks - 1) {
        atomicExch(bar, 0u);
        __threadfence();
        atomicAdd(bar + 1, 1u);
      } else {
        long long spins = 0;
        while (*vgen == g) {
          if (++spins > spin_limit) { atomicExch(status, MAK_ERR_TIMEOUT); ok = 0; break; }
          if (*((volatile int*)status) == MAK_ERR_TIMEOUT) { ok = 0; break; }
          __nanosleep(64);
        }
      }
      __threadfence();
    }
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// Barrier of the CTAs that factor one panel together.  SYNC_GRID: the
// bounded global barrier above, inside a cooperative launch (any number of
// co-resident CTAs).  SYNC_CLUSTER: the hardware barrier of a thread-block
// cluster (all of the panel's CTAs form one cluster of at most 8): its
// arrive.release / wait.acquire pair orders every write of the CTAs (global
// memory included) before the reads that follow it in the other CTAs, with
// no polling of global memory.  It needs no bound: the kernels that use it
// take the same branches in every CTA, so every thread of the cluster
// arrives.  Unlike a cooperative launch, cluster launches of different
// streams run side by side.
//
// SYNC_HIER: a cooperative grid made of clusters (launched with both the
// cooperative and the cluster attribute).  The CTAs of a cluster meet at
// the cluster barrier and only the clusters' first CTAs meet at the bounded
// global barrier (`nblocks` = the number of clusters), then release their
// clusters with a second cluster barrier: far fewer arrivals on the global
// counter, and the panels can combine a cluster's partials through
// distributed shared memory before the global round.  On a timeout every
// CTA of a cluster learns it from its cluster's flag after the last cluster
// barrier (no CTA is left waiting at a cluster barrier).
enum { SYNC_GRID = 0, SYNC_CLUSTER = 1, SYNC_HIER = 2 };
__device__ __forceinline__ unsigned cluster_ctarank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned cluster_nctarank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::
                   : "memory");
}
// the second half of a SYNC_HIER barrier: the clusters' first CTAs meet at
// the global barrier, record its outcome in their cluster's flag and
// release their clusters; every CTA of a cluster then reads the same flag,
// so a cluster always takes one branch (a CTA that left while the others
// went on to the next cluster barrier would leave them waiting for good)
__device__ __forceinline__ bool hier_leader_barrier(unsigned* bar, unsigned nclusters, int* status,
                                                    int* cluster_flag) {
  if (cluster_ctarank() == 0) {
    const bool ok = grid_barrier(bar, nclusters, status);
    if (threadIdx.x == 0) *(volatile int*)cluster_flag = ok ? 1 : 0;
  }
  cluster_sync_all();
  return __ldcg(cluster_flag) != 0;
}
template <int SYNC>
__device__ __forceinline__ bool panel_sync(unsigned* bar, unsigned nblocks, int* status,
                                           int* cluster_flag = nullptr) {
  if constexpr (SYNC == SYNC_CLUSTER) {
    cluster_sync_all();
    return true;
  } else if constexpr (SYNC == SYNC_HIER) {
    cluster_sync_all();
    return hier_leader_barrier(bar, nblocks, status, cluster_flag);
  } else {
    return grid_barrier(bar, nblocks, status);
  }
}
// largest cluster the panels use (the portable limit)
constexpr int kPanelClusterMax = 8;

// Loads from the shared memory of CTA `rank` of the calling thread's
// cluster (distributed shared memory): `p` is the address of the same
// variable in the caller's own shared memory.  Used by the cluster variant
// of the panels to read the other CTAs' partials after the cluster barrier
// instead of a round trip through L2.
__device__ __forceinline__ uint32_t dsmem_addr(const void* p, unsigned rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;"
               : "=r"(r)
               : "r"((uint32_t)__cvta_generic_to_shared(p)), "r"(rank));
  return r;
}
__device__ __forceinline__ double dsmem_ld(const double* p, unsigned rank) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(dsmem_addr(p, rank)) : "memory");
  return v;
}
__device__ __forceinline__ float dsmem_ld(const float* p, unsigned rank) {
  float v;
  asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(dsmem_addr(p, rank)) : "memory");
  return v;
}
__device__ __forceinline__ int dsmem_ld(const int* p, unsigned rank) {
  int v;
  asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(dsmem_addr(p, rank)) : "memory");
  return v;
}
template <class R>
__device__ __forceinline__ cplx<R> dsmem_ld(const cplx<R>* p, unsigned rank) {
  return {dsmem_ld(&p->re, rank), dsmem_ld(&p->im, rank)};
}

// --------------------------------------------------------------- host side --
#define MAK_CUDA_TRY(expr)                         \
  do {                                             \
    cudaError_t e_ = (expr);                       \
    if (e_ != cudaSuccess) return MAK_ERR_CUDA;    \
  } while (0)

#define MAK_TRY(expr)          \
  do {                         \
    int r_ = (expr);           \
    if (r_ != 0) return r_;    \
  } while (0)

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Host state that is set up lazily (device attributes, kernel attributes,
// streams, events) belongs to ONE device: a process may drive several GPUs
// (one per Julia task or host thread), and a kernel attribute set, or a
// stream created, while device 0 was current does not carry over to
// device 1.  Such state is kept per device, indexed by cudaGetDevice() at
// the call.
constexpr int kMaxDevices = 64;
inline int current_device() {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= kMaxDevices) d = 0;
  return d;
}
// One value per device, computed once per device by `init` (run with that
// device current; concurrent first calls on one device wait for it).
template <class V>
struct PerDevice {
  std::once_flag flag[kMaxDevices];
  V val[kMaxDevices] = {};
  template <class F>
  V get(F&& init) {
    const int d = current_device();
    std::call_once(flag[d], [&] { val[d] = init(); });
    return val[d];
  }
};

// Bump allocator over the caller's workspace.  With base == nullptr it only
// measures (used by the *_workspace queries, LAPACK's lwork = -1 pattern).
struct Arena {
  char* base;
  size_t cap;
  size_t off = 0;
  Arena(void* b, size_t c) : base((char*)b), cap(c) {}
  template <class T>
  T* take(size_t count) {
    // align the absolute address (offsets alone when only measuring)
    size_t addr = (size_t)base + off;
    off += align_up(addr, 256) - addr;
    T* p = base ? (T*)(base + off) : nullptr;
    off += count * sizeof(T);
    return p;
  }
  bool ok() const { return base == nullptr || off <= cap; }
};

int num_sms();
int max_smem_optin();

// process-wide count of kernels this library has launched (mak_kernel_launches)
std::atomic<unsigned long long>& launch_counter();
inline void note_launch() { launch_counter().fetch_add(1, std::memory_order_relaxed); }

// Device-side stop of a fixed-iteration loop.  While a flag is installed for
// the calling host thread (SkipScope), the library's heavy kernels launched
// from that thread take the flag's address and return at once when it is
// non-zero; the loop's convergence test sets it on the device, so converged
// iterations cost only their launches and need no host synchronization.
inline const int*& skip_flag_slot() {
  static thread_local const int* p = nullptr;
  return p;
}
inline const int* skip_flag() { return skip_flag_slot(); }
struct SkipScope {
  const int* prev;
  explicit SkipScope(const int* f) : prev(skip_flag_slot()) { skip_flag_slot() = f; }
  ~SkipScope() { skip_flag_slot() = prev; }
  SkipScope(const SkipScope&) = delete;
  SkipScope& operator=(const SkipScope&) = delete;
};
__device__ __forceinline__ bool skipped(const int* f) {
  return f != nullptr && *(const volatile int*)f != 0;
}

// kernel classes timed by the optional profiler (mak_profile_*)
enum ProfKind {
  PROF_GEMM_NATIVE = 0,  // SIMT FP64/FP32 GEMM (work = flops)
  PROF_GEMM_MIXED = 1,   // split-precision tensor-core GEMM (work = fp64-equivalent flops)
  PROF_QR_PANEL = 2,     // cooperative Householder panel (work = bytes)
  PROF_GJ_PANEL = 3      // cooperative Gauss-Jordan panel (work = bytes)
};
// RAII: records an event pair around the launches in its scope when the
// profiler is on; a no-op otherwise.
struct ProfScope {
  cudaEvent_t e0 = nullptr;
  cudaStream_t st;
  int kind;
  double work;
  ProfScope(cudaStream_t s, int k, double w);
  ~ProfScope();
};

}  // namespace mak
