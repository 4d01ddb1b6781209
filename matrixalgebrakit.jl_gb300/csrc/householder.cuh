// Householder reflector scalars and the column-norm helpers shared by the
// multi-CTA QR panel (qr.cu) and the single-CTA small-block QR (small.cu).
#pragma once
#include "mak_common.cuh"

namespace mak {

// Column norms in the panel: a plain sum of squares (one FMA per element on
// the FP64 pipe, which GB300 runs at about 1.6 DFMA per clock per SM) next to
// the largest magnitude, compared as IEEE bits on the integer pipe.  When the
// largest magnitude lies outside [2^lo, 2^hi] the squares could overflow or
// lose precision, and the norm is recomputed from values scaled by a power
// of two (a second, rarely taken pass).
template <class R> struct NormKey;
template <> struct NormKey<double> {
  using K = unsigned long long;
  static constexpr int lo = -500, hi = 500;
  __device__ static K key(double x) {
    return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
  }
  __device__ static double val(K k) { return __longlong_as_double((long long)k); }
};
template <> struct NormKey<float> {
  using K = unsigned;
  static constexpr int lo = -50, hi = 50;
  __device__ static K key(float x) { return __float_as_uint(x) & 0x7FFFFFFFu; }
  __device__ static float val(K k) { return __uint_as_float(k); }
};
template <class R> __device__ __forceinline__ typename NormKey<R>::K mag_key(R x) {
  return NormKey<R>::key(x);
}
template <class R> __device__ __forceinline__ typename NormKey<R>::K mag_key(cplx<R> x) {
  const auto a = NormKey<R>::key(x.re), b = NormKey<R>::key(x.im);
  return a > b ? a : b;
}
__device__ __forceinline__ bool finite_(double x) { return isfinite(x); }
__device__ __forceinline__ bool finite_(float x) { return isfinite(x); }
template <class R> __device__ __forceinline__ bool finite_(cplx<R> x) {
  return isfinite(x.re) && isfinite(x.im);
}
template <class R> __device__ __forceinline__ R sq_add(R s, R x) { return fma_(x, x, s); }
template <class R> __device__ __forceinline__ R sq_add(R s, cplx<R> x) {
  return fma_(x.re, x.re, fma_(x.im, x.im, s));
}
template <class R> __device__ __forceinline__ void ssq_scaled_add(R& s, R x, R scale) {
  const R y = x * scale;
  s = fma_(y, y, s);
}
template <class R> __device__ __forceinline__ void ssq_scaled_add(R& s, cplx<R> x, R scale) {
  ssq_scaled_add(s, x.re, scale);
  ssq_scaled_add(s, x.im, scale);
}
template <class K> __device__ __forceinline__ K warp_max_key(K v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const K w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}
// 0: the plain sum of squares is accurate; 1: rescale first
template <class R> __device__ __forceinline__ int norm_needs_rescale(typename NormKey<R>::K m) {
  using NK = NormKey<R>;
  if (m == 0) return 0;
  const R v = NK::val(m);
  if (!(v < R(INFINITY))) return 0;  // Inf / NaN propagate through the plain sum
  return (v < ldexp(R(1), NK::lo) || v > ldexp(R(1), NK::hi)) ? 1 : 0;
}

// beta / tau / 1/(alpha-beta) of one reflector, LAPACK ?larfg convention:
// H^H [alpha; x] = [beta; 0], H = I - tau v v^H, v = [1; x/(alpha-beta)].
// One reciprocal of beta, one of alpha - beta (|.|^2 for complex) and one
// square root; values are scaled by exact powers of two, and magnitudes near
// the ends of the exponent range take the IEEE operations.
template <class T>
__device__ __forceinline__ void larfg_scalars(T alpha, real_t<T> xnorm, T& beta, T& tau, T& scal) {
  using R = real_t<T>;
  R ar = re_(alpha), ai = im_(alpha);
  if (xnorm == R(0) && ai == R(0)) {
    tau = zero_<T>();
    beta = alpha;
    scal = one_<T>();
    return;
  }
  const R w = fmax(fmax(fabs(ar), fabs(ai)), xnorm);
  const int ew = exp2_of(w);
  const int lim = sizeof(R) == 8 ? 1000 : 100;
  if (ew < -lim + 4 || ew > lim - 4) {
    R nrm = w * sqrt((ar / w) * (ar / w) + (ai / w) * (ai / w) + (xnorm / w) * (xnorm / w));
    R b = ar >= R(0) ? -nrm : nrm;
    beta = make_scalar<T>(b, 0);
    tau = make_scalar<T>((b - ar) / b, -ai / b);
    scal = inv_(alpha - beta);
    return;
  }
  const R sd = pow2_(R(0), -ew), su = pow2_(R(0), ew);  // exact scalings
  const R a1 = ar * sd, a2 = ai * sd, a3 = xnorm * sd;
  const R nrm = sqrt_nr(fma_(a1, a1, fma_(a2, a2, a3 * a3))) * su;
  const R b = ar >= R(0) ? -nrm : nrm;
  const R rb = rcp_nr(b);
  beta = make_scalar<T>(b, 0);
  tau = make_scalar<T>((b - ar) * rb, -ai * rb);
  // alpha - beta = (ar - b, ai) with |ar - b| = |ar| + nrm >= nrm
  const R zr = ar - b;
  if constexpr (traits<T>::cpx) {
    const R z1 = zr * sd, z2 = ai * sd;  // |z| in [2^-1, 4) after scaling by w
    const R d = rcp_nr(fma_(z1, z1, z2 * z2)) * sd;
    scal = make_scalar<T>(z1 * d, -z2 * d);
  } else {
    scal = make_scalar<T>(rcp_nr(zr), 0);
  }
}

// The same scalars from the sum of squares ssq = |x|^2 and the largest
// component magnitude amax of x, without forming |x| first: |beta| =
// sqrt(|alpha|^2 + ssq) is one square root, which saves a whole Newton
// chain on the column's critical path.  Scaling by w = max(|alpha|, amax)
// (a power of two) keeps the scaled sum within [1, 2 (n + 1)].
template <class T>
__device__ __forceinline__ void larfg_scalars_ssq(T alpha, real_t<T> ssq, real_t<T> amax, T& beta, T& tau,
                                  T& scal) {
  using R = real_t<T>;
  const R ar = re_(alpha), ai = im_(alpha);
  const R w = fmax(fmax(fabs(ar), fabs(ai)), amax);
  const int ew = exp2_of(w);
  const int lim = sizeof(R) == 8 ? 1000 : 100;
  if (ssq == R(0) || !(w > R(0)) || ew < -lim + 4 || ew > lim - 4) {
    larfg_scalars(alpha, sqrt_nr_safe(ssq), beta, tau, scal);
    return;
  }
  const R sd = pow2_(R(0), -ew), su = pow2_(R(0), ew);  // exact scalings
  const R a1 = ar * sd, a2 = ai * sd;
  const R s3 = (ssq * sd) * sd;
  const R nrm = sqrt_nr(fma_(a1, a1, fma_(a2, a2, s3))) * su;
  const R b = ar >= R(0) ? -nrm : nrm;
  const R rb = rcp_nr(b);
  beta = make_scalar<T>(b, 0);
  tau = make_scalar<T>((b - ar) * rb, -ai * rb);
  const R zr = ar - b;
  if constexpr (traits<T>::cpx) {
    const R z1 = zr * sd, z2 = ai * sd;
    const R d = rcp_nr(fma_(z1, z1, z2 * z2)) * sd;
    scal = make_scalar<T>(z1 * d, -z2 * d);
  } else {
    scal = make_scalar<T>(rcp_nr(zr), 0);
  }
}

}  // namespace mak
