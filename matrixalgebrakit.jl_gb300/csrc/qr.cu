// Blocked Householder QR with positive-diagonal gauge, GB300 native.
//
// Replaces the reference's LAPACK/cuSOLVER path
//   qr_householder!  (src/implementations/qr.jl:132-188)
//   = geqrt!/geqrf!  (panel + T factor, src/yalapack.jl:303-333 / 168-199)
//   + gemqrt!/unmqr! on one!(Q)  (Q formation, src/yalapack.jl:882-927)
//   + uppertriangular! R copy   (src/common/initialization.jl:18-26)
//   + gaugefix!(qr_householder!) (src/common/gauge.jl:16-25, sign_safe
//     src/common/safemethods.jl:10-11)
//
// Structure on the device, per panel of jb <= 32 columns starting at j0:
//  1. qr_panel_kernel: ONE launch factors the (m-j0) x jb panel: a
//     thread-block cluster of up to 8 CTAs for panels of up to 8 x 256 rows
//     (hardware cluster barrier; clusters of different streams run side by
//     side, which the batched driver relies on), a cooperative grid of up to
//     one CTA per SM beyond that (bounded global barrier).
//     Each CTA keeps a contiguous slab of panel rows resident in shared
//     memory for the whole panel; a column costs one barrier:
//     the reflector norm and the dot products of the still unscaled column
//     with the columns to its right are published together, and w = v^H A
//     follows from them once beta/tau are known.  Norms are plain sums of
//     squares with a rescaled two-round path when the largest magnitude is
//     outside a safe range, and every cross-CTA reduction is done in a fixed
//     order, so all CTAs derive bit-identical beta/tau/w.  The panel's Gram
//     matrix V^H V is reduced at the end and the CTAs form the T factor's
//     columns (forward, column-wise larft recurrence).
//  2. larfb on the trailing columns:  W = V^H C (split-K GEMM, V read in
//     place through a unit-lower mask), W2 = T^H W (reduce_trmm_kernel),
//     C -= V W2 (GEMM).
// Q is then accumulated backwards (orgqr order, exploiting the identity
// structure: block b only touches Q[j0:, j0:]) starting from [diag(s); 0]
// where s = sign_safe(diag R): the gauge fix Q <- Q diag(s) is folded into the
// starting matrix because Q diag(s) = H_1...H_k [diag(s); 0].  R is written
// once, already multiplied by conj(s) row-wise.
#include "gemm.cuh"
#include "householder.cuh"
#include "internal.h"

#include <cstdlib>
#include <mutex>

namespace mak {

constexpr int NBMAX = 32;      // widest panel handled by one cooperative launch
constexpr int PANEL_THREADS = 256;

template <class T>
struct PanelArgs {
  T* A;                 // panel (row j0, col j0) of the packed matrix
  int64_t lda;
  int mp;               // panel rows
  int jb;               // panel columns
  int rpc;              // panel rows owned by one CTA
  T* tau;               // [jb]
  T* Tm;                // [NBMAX x NBMAX], ld NBMAX
  real_t<T>* part_nrm;  // [2][3][gstride] by round parity (sums of squares, largest
                        // magnitudes of columns j and j+1), then [gstride] rescaled sums
  T* part_w;            // [2][gstride][NBMAX] dot partials by round parity, then
                        // [gstride][NBMAX] for the rescaled path, then
                        // [2][gstride][NBMAX] column j+1's dot partials (pair rounds)
  T* part_g;            // [G][NBMAX*NBMAX]
  T* alpha_buf;         // [2][NBMAX]: row j of the panel by round parity, then
                        // [2][NBMAX] row j+1 (pair rounds)
  T* gram;              // [NBMAX*NBMAX]: the panel's reduced Gram matrix V^H V
  unsigned* bar;        // grid barrier words
  int* cflag;           // [gstride] outcome of the last global round, per cluster (SYNC_HIER)
  int* status;
  int gstride;          // allocation stride of the per-CTA partial rows
  int pair;             // two columns per barrier round where the norms allow
};

template <class T, int SYNC>
__global__ void __launch_bounds__(PANEL_THREADS, SYNC == SYNC_CLUSTER ? 2 : 1)
qr_panel_kernel(PanelArgs<T> a) {
  using R = real_t<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* Ps = reinterpret_cast<T*>(smem_raw);  // rpc x jb, column-major, ld = ldp
  __shared__ R red_r[32];
  __shared__ typename NormKey<R>::K red_k[32];
  __shared__ typename NormKey<R>::K red_k2[32];
  __shared__ R sc_r[3];
  __shared__ int sc_flag, sc_flag2, sc_pair;
  __shared__ T wsh[NBMAX], wsh1[NBMAX];
  __shared__ T red_w[PANEL_THREADS / 32][NBMAX];
  __shared__ T red_g[PANEL_THREADS / 32][NBMAX];  // pair rounds: column j+1's dots
  __shared__ T sc[3], sc1[3];
  __shared__ T rowj[NBMAX], rowj1[NBMAX];
  // cluster variant: this CTA's published partials of the current column
  // (by column parity), read by the other CTAs through distributed shared
  // memory after the cluster barrier
  __shared__ R x_nrm[2][3];       // sum of squares, largest magnitude (of column j+1 too)
  __shared__ T x_w[2][NBMAX];     // dot partials
  __shared__ T x_g[2][NBMAX];     // pair rounds: column j+1's dot partials
  __shared__ T x_row[2][NBMAX];   // row j (the CTA that holds it)
  __shared__ T x_row1[2][NBMAX];  // pair rounds: row j+1
  constexpr bool kCl = SYNC == SYNC_CLUSTER;
  constexpr bool kH = SYNC == SYNC_HIER;
  constexpr bool kSm = kCl || kH;  // partials published in shared memory first
  const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
  // hierarchical grid: C CTAs per cluster, H clusters; the global round
  // then carries one partial row per cluster
  const int C = kH ? (int)cluster_nctarank() : 1;
  const int H = G / C;
  const unsigned nsync = kH ? (unsigned)H : (unsigned)G;
  int* const cflag = kH ? a.cflag + b / C : nullptr;
  const int lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  const int rpc = a.rpc, jb = a.jb;
  const int ldp = rpc | 1;  // slab leading dimension (odd: conflict-free column strides)
  const int r0 = b * rpc;
  const int nr = max(0, min(a.mp, r0 + rpc) - r0);

  for (int c = 0; c < jb; c++)
    for (int r = tid; r < nr; r += blockDim.x) Ps[r + c * ldp] = a.A[(r0 + r) + (int64_t)c * a.lda];
  __syncthreads();

  // Per column one grid-wide reduction: the partial sums of squares of x =
  // column j below the diagonal, its largest magnitude, the partial dot
  // products d_c = sum_{r>j} conj(x_r) A[r, c] of the still unscaled x with
  // the columns c > j, and row j, all published in one round.  Since
  // v = [1; scal x], w_c = v^H A[:, c] = A[j, c] + conj(scal) d_c follows
  // once larfg has fixed scal, without a second round.  The partials are
  // double-buffered by column parity: a CTA writes column j+1's slot only
  // after every CTA passed barrier j, i.e. finished reading column j-1's.
  // A column whose largest magnitude lies outside [2^lo, 2^hi] takes the
  // rescaled two-round path instead (the same decision in every CTA).
  // Pair rounds (pair_mode): one round publishes, next to column j's
  // partials, the dot products of column j+1 below row j+1 with the columns
  // c > j and row j+1.  Since H_j is unitary, column j+1's sum of squares
  // and dot products after the reflection follow from those Gram entries,
  // H_j's scalars and rows j, j+1, so column j+1's reflector is formed in
  // the same round (a rank-2 update follows).  When that derivation would
  // cancel (column j+1 keeps less than half of its norm below row j+1) or
  // a magnitude is outside the safe range, column j+1 takes its own round
  // instead; the test sees the same numbers in every CTA.
  const bool pair_mode = !kH && a.pair != 0;
  for (int j = 0, rnd = 0; j < jb; rnd++) {
    T* col = Ps + j * ldp;
    T* col1 = col + ldp;  // column j+1 (pair rounds)
    const int par = rnd & 1;
    const bool two = pair_mode && j + 1 < jb;
    R* pn = a.part_nrm + (int64_t)par * 3 * a.gstride;
    T* pw = a.part_w + (int64_t)par * a.gstride * NBMAX;
    T* pwg = a.part_w + (int64_t)(3 + par) * a.gstride * NBMAX;
    T* prow = a.alpha_buf + par * NBMAX;
    T* prow1 = a.alpha_buf + (2 + par) * NBMAX;
    using NK = NormKey<R>;
    using Key = typename NK::K;
    const int rs = max(0, j + 1 - r0);  // first local row below the diagonal
    const int jy = j + 1 - r0;          // local index of row j+1
    // ---- phase A: warp w takes a slice of this CTA's rows below the
    // diagonal; lane c >= j accumulates conj(x_r) A[r, c] over the slice
    // (lane j: conj(x_r) x_r, the sum of squares) and the largest magnitude
    // of x (pair rounds: also conj(y_r) A[r, c] for y = column j+1 below row
    // j+1, and y's largest magnitude).  No cross-lane reductions (GB300
    // issues about two FP64 operations per clock per SM, so butterflies over
    // 32 lanes would cost more than the products); warp 0 adds the eight
    // slices.  The slab's odd leading dimension keeps the column-strided
    // reads conflict-free.
    {
      const int nx = nr - rs;
      const int per = nx > 0 ? (nx + nw - 1) / nw : 0;
      const int ra = rs + wid * per, rb = min(nr, ra + per);
      T s0 = zero_<T>(), s1 = zero_<T>(), g0 = zero_<T>(), g1 = zero_<T>();
      Key mk = 0, mk2 = 0;
      if (lane >= j && lane < jb) {
        const T* pc = Ps + lane * ldp;
        int r = ra;
        if (two) {
          for (; r + 1 < rb; r += 2) {
            const T x0 = col[r], x1 = col[r + 1];
            const T y0 = r == jy ? zero_<T>() : col1[r];
            const T y1 = r + 1 == jy ? zero_<T>() : col1[r + 1];
            const T c0 = pc[r], c1 = pc[r + 1];
            s0 = fma_(conj_(x0), c0, s0);
            s1 = fma_(conj_(x1), c1, s1);
            g0 = fma_(conj_(y0), c0, g0);
            g1 = fma_(conj_(y1), c1, g1);
            const Key k0 = mag_key(x0), k1 = mag_key(x1);
            const Key k = k0 > k1 ? k0 : k1;
            mk = k > mk ? k : mk;
            const Key q0 = mag_key(y0), q1 = mag_key(y1);
            const Key q = q0 > q1 ? q0 : q1;
            mk2 = q > mk2 ? q : mk2;
          }
          if (r < rb) {
            const T x0 = col[r];
            const T y0 = r == jy ? zero_<T>() : col1[r];
            const T c0 = pc[r];
            s0 = fma_(conj_(x0), c0, s0);
            g0 = fma_(conj_(y0), c0, g0);
            const Key k = mag_key(x0);
            mk = k > mk ? k : mk;
            const Key q = mag_key(y0);
            mk2 = q > mk2 ? q : mk2;
          }
        } else {
          for (; r + 1 < rb; r += 2) {
            const T x0 = col[r], x1 = col[r + 1];
            s0 = fma_(conj_(x0), pc[r], s0);
            s1 = fma_(conj_(x1), pc[r + 1], s1);
            const Key k0 = mag_key(x0), k1 = mag_key(x1);
            const Key k = k0 > k1 ? k0 : k1;
            mk = k > mk ? k : mk;
          }
          if (r < rb) {
            const T x0 = col[r];
            s0 = fma_(conj_(x0), pc[r], s0);
            const Key k = mag_key(x0);
            mk = k > mk ? k : mk;
          }
        }
      }
      red_w[wid][lane] = s0 + s1;
      if (two) red_g[wid][lane] = g0 + g1;
      if (lane == j) {
        red_k[wid] = mk;
        red_k2[wid] = mk2;
      }
    }
    if (j >= r0 && j < r0 + nr)
      for (int c = j + tid; c < jb; c += blockDim.x) {
        if constexpr (kSm) x_row[par][c] = Ps[(j - r0) + c * ldp];
        else prow[c] = Ps[(j - r0) + c * ldp];
      }
    if (two && jy >= 0 && jy < nr)
      for (int c = j + tid; c < jb; c += blockDim.x) {
        if constexpr (kSm) x_row1[par][c] = Ps[jy + c * ldp];
        else prow1[c] = Ps[jy + c * ldp];
      }
    __syncthreads();
    if (wid == 0) {
      T s = zero_<T>();
      for (int w = 0; w < nw; w++) s += red_w[w][lane];
      if (lane > j && lane < jb) {
        if constexpr (kSm) x_w[par][lane] = s;
        else pw[(int64_t)b * NBMAX + lane] = s;
      }
      if (two) {
        T sg = zero_<T>();
        for (int w = 0; w < nw; w++) sg += red_g[w][lane];
        if (lane > j && lane < jb) {
          if constexpr (kSm) x_g[par][lane] = sg;
          else pwg[(int64_t)b * NBMAX + lane] = sg;
        }
      }
      if (lane == j) {
        Key m = 0, m2 = 0;
        for (int w = 0; w < nw; w++) {
          m = red_k[w] > m ? red_k[w] : m;
          m2 = red_k2[w] > m2 ? red_k2[w] : m2;
        }
        if constexpr (kSm) {
          x_nrm[par][0] = re_(s);
          x_nrm[par][1] = NK::val(m);
          x_nrm[par][2] = NK::val(m2);
        } else {
          pn[b] = re_(s);
          pn[a.gstride + b] = NK::val(m);
          pn[2 * a.gstride + b] = NK::val(m2);
        }
      }
    }
    if constexpr (kH) {
      // the cluster's first CTA combines its C CTAs' partials (rank order)
      // and publishes one row per cluster for the global round
      cluster_sync_all();
      if (cluster_ctarank() == 0) {
        const int h = b / C;
        if (wid == 0) {
          if (lane == j) {
            R s2 = R(0);
            Key m2 = 0;
            for (int r = 0; r < C; r++) {
              s2 += dsmem_ld(&x_nrm[par][0], (unsigned)r);
              const Key k = NK::key(dsmem_ld(&x_nrm[par][1], (unsigned)r));
              m2 = k > m2 ? k : m2;
            }
            pn[h] = s2;
            pn[a.gstride + h] = NK::val(m2);
          }
          if (lane > j && lane < jb) {
            T s2 = zero_<T>();
            for (int r = 0; r < C; r++) s2 += dsmem_ld(&x_w[par][lane], (unsigned)r);
            pw[(int64_t)h * NBMAX + lane] = s2;
          }
        }
        const int own = j / rpc;  // the CTA holding row j
        if (own / C == h && wid == 1 && lane >= j && lane < jb)
          prow[lane] = dsmem_ld(&x_row[par][lane], (unsigned)(own % C));
      }
      if (!hier_leader_barrier(a.bar, nsync, a.status, cflag)) return;
    } else {
      if (!panel_sync<SYNC>(a.bar, G, a.status)) return;
    }

    // ---- phase B: every CTA combines the partials in the same fixed order
    // and so derives bit-identical beta / tau / w.  Warp 0: the norm; every
    // warp: a slice of the CTAs' dot partials (lane = column); lane j of
    // warp 1 (or of warp 0 with one warp): row j; warp 2: row j+1.
    const int NP = kH ? H : G;  // partial rows to combine
    if (wid == 0) {
      R s = R(0);
      Key m = 0, m2 = 0;
      for (int q = lane; q < NP; q += 32) {
        if constexpr (kCl) {
          s += dsmem_ld(&x_nrm[par][0], (unsigned)q);
          const Key k = NK::key(dsmem_ld(&x_nrm[par][1], (unsigned)q));
          m = k > m ? k : m;
          if (two) {
            const Key k2 = NK::key(dsmem_ld(&x_nrm[par][2], (unsigned)q));
            m2 = k2 > m2 ? k2 : m2;
          }
        } else {
          s += ld_cg(&pn[q]);
          const Key k = NK::key(ld_cg(&pn[a.gstride + q]));
          m = k > m ? k : m;
          if (two) {
            const Key k2 = NK::key(ld_cg(&pn[2 * a.gstride + q]));
            m2 = k2 > m2 ? k2 : m2;
          }
        }
      }
      s = warp_sum(s);
      m = warp_max_key(m);
      if (two) m2 = warp_max_key(m2);
      if (lane == 0) {
        sc_r[0] = s;
        sc_r[1] = NK::val(m);
        sc_flag = norm_needs_rescale<R>(m);
        sc_flag2 = norm_needs_rescale<R>(m2);
      }
    }
    {
      const int per = (NP + nw - 1) / nw;
      const int q0 = wid * per, q1 = min(NP, q0 + per);
      T a0 = zero_<T>(), a1 = zero_<T>(), a2 = zero_<T>(), a3 = zero_<T>();
      T b0 = zero_<T>(), b1 = zero_<T>(), b2 = zero_<T>(), b3 = zero_<T>();
      if (lane > j && lane < jb) {
        int q = q0;
        if constexpr (kCl) {
          for (; q < q1; q++) {
            a0 += dsmem_ld(&x_w[par][lane], (unsigned)q);
            if (two) b0 += dsmem_ld(&x_g[par][lane], (unsigned)q);
          }
        } else {
          for (; q + 3 < q1; q += 4) {
            a0 += ld_cg(&pw[(int64_t)q * NBMAX + lane]);
            a1 += ld_cg(&pw[(int64_t)(q + 1) * NBMAX + lane]);
            a2 += ld_cg(&pw[(int64_t)(q + 2) * NBMAX + lane]);
            a3 += ld_cg(&pw[(int64_t)(q + 3) * NBMAX + lane]);
            if (two) {
              b0 += ld_cg(&pwg[(int64_t)q * NBMAX + lane]);
              b1 += ld_cg(&pwg[(int64_t)(q + 1) * NBMAX + lane]);
              b2 += ld_cg(&pwg[(int64_t)(q + 2) * NBMAX + lane]);
              b3 += ld_cg(&pwg[(int64_t)(q + 3) * NBMAX + lane]);
            }
          }
          for (; q < q1; q++) {
            a0 += ld_cg(&pw[(int64_t)q * NBMAX + lane]);
            if (two) b0 += ld_cg(&pwg[(int64_t)q * NBMAX + lane]);
          }
        }
      }
      red_w[wid][lane] = (a0 + a1) + (a2 + a3);
      if (two) red_g[wid][lane] = (b0 + b1) + (b2 + b3);
    }
    if (wid == (nw > 1 ? 1 : 0) && lane >= j && lane < jb) {
      // row j is held by the CTA whose rows contain j
      if constexpr (kCl) rowj[lane] = dsmem_ld(&x_row[par][lane], (unsigned)(j / rpc));
      else rowj[lane] = ld_cg(&prow[lane]);
    }
    if (two && wid == (nw > 2 ? 2 : 0) && lane >= j && lane < jb) {
      if constexpr (kCl) rowj1[lane] = dsmem_ld(&x_row1[par][lane], (unsigned)((j + 1) / rpc));
      else rowj1[lane] = ld_cg(&prow1[lane]);
    }
    __syncthreads();
    const bool rescale = sc_flag != 0;
    if (two && !rescale) {
      // ---- both reflectors on warp 0 (every lane derives the scalars, lane
      // c the column-c quantities).  H_j: f_c = conj(tau) w_c as below.
      // Column j+1 after H_j^H: with v = [1; scal x] and x_1 = A[j+1, j],
      //   p_c = sum_{r>j+1} conj(v_r) A[r, c] = conj(scal) (d_c - conj(x_1) A[j+1, c])
      //   q   = sum_{r>j+1} |v_r|^2 = |scal|^2 (|x|^2 - |x_1|^2)
      //   G_c = sum_{r>j+1} conj(A'[r, j+1]) A'[r, c]
      //       = g_c - conj(p_{j+1}) f_c - conj(f_{j+1}) p_c + conj(f_{j+1}) f_c q
      //   A'[j+1, c] = A[j+1, c] - scal x_1 f_c,
      // and column j+1's reflector follows from alpha = A'[j+1, j+1] and the
      // sum of squares G_{j+1}, with d'_c = G_c (c > j+1).
      if (wid == 0) {
        T d = zero_<T>(), g = zero_<T>();
        for (int w = 0; w < nw; w++) {
          d += red_w[w][lane];
          g += red_g[w][lane];
        }
        T beta, tau, scal;
        larfg_scalars_ssq(rowj[j], sc_r[0], sc_r[1], beta, tau, scal);
        const bool act = lane > j && lane < jb;
        const T f = act ? conj_(tau) * fma_(conj_(scal), d, rowj[lane]) : zero_<T>();
        const T x1 = rowj1[j];
        const T v1 = x1 * scal;
        const T p = act ? conj_(scal) * fma_(-conj_(x1), rowj1[lane], d) : zero_<T>();
        const R q = abs2_(scal) * (sc_r[0] - abs2_(x1));
        const T f1 = shfl_idx_(f, j + 1), p1 = shfl_idx_(p, j + 1);
        const T gp = act ? (g - conj_(p1) * f - conj_(f1) * p) + (conj_(f1) * f) * q : zero_<T>();
        const T r1 = act ? fma_(-v1, f, rowj1[lane]) : zero_<T>();
        const R ssq1 = re_(shfl_idx_(gp, j + 1));
        const T alpha1 = shfl_idx_(r1, j + 1);
        const R nrm1 = re_(shfl_idx_(g, j + 1)) + abs2_(rowj1[j + 1]) + abs2_(rowj[j + 1]);
        const bool fin = __all_sync(0xffffffffu, !act || (finite_(gp) && finite_(r1)));
        const int en = exp2_of(nrm1);
        const int lim = sizeof(R) == 8 ? 1000 : 100;
        const bool ok = fin && sc_flag2 == 0 && en > -lim && en < lim && ssq1 >= R(0.5) * nrm1;
        T beta1 = zero_<T>(), tau1 = zero_<T>(), scal1 = one_<T>(), f2 = zero_<T>();
        if (ok) {
          // a power of two within a factor 2 sqrt(2) of sqrt(ssq1) scales the
          // square root in place of column j+1's largest magnitude
          const R prox = ssq1 > R(0) ? pow2_(R(0), exp2_of(ssq1) >> 1) : R(0);
          larfg_scalars_ssq(alpha1, ssq1, prox, beta1, tau1, scal1);
          if (lane > j + 1 && lane < jb) f2 = conj_(tau1) * fma_(conj_(scal1), gp, r1);
        }
        wsh[lane] = f;
        wsh1[lane] = f2;
        if (lane == 0) {
          sc[0] = beta;
          sc[1] = tau;
          sc[2] = scal;
          sc1[0] = beta1;
          sc1[1] = tau1;
          sc1[2] = scal1;
          sc_pair = ok ? 1 : 0;
        }
      }
      __syncthreads();
      const T beta = sc[0], tau = sc[1], scal = sc[2];
      const bool ok = sc_pair != 0;
      if (b == 0 && tid == 0) {
        a.tau[j] = tau;
        if (ok) a.tau[j + 1] = sc1[1];
      }
      const int rj = max(0, j - r0);
      if (ok) {
        // column j: scale to v; column j+1: apply H_j^H, then scale below
        // row j+1 to v' (row j+1 becomes beta')
        const T f1 = wsh[j + 1], scal1 = sc1[2];
        for (int r = rj + tid; r < nr; r += blockDim.x) {
          const int gr = r0 + r;
          T v = one_<T>();
          if (gr > j) {
            v = col[r] * scal;
            col[r] = v;
          }
          const T y = fma_(-v, f1, col1[r]);
          col1[r] = gr > j + 1 ? y * scal1 : y;
        }
        __syncthreads();
        // rank-2 update of the columns c > j+1: rows >= j take v f_c, rows
        // >= j+1 also v' f'_c (v_j = 1, v'_{j+1} = 1)
        for (int c = j + 2 + wid; c < jb; c += nw) {
          const T fa = wsh[c], fb = wsh1[c];
          T* pc = Ps + c * ldp;
          for (int r = rj + lane; r < nr; r += 32) {
            const int gr = r0 + r;
            const T v = gr == j ? one_<T>() : col[r];
            T y = fma_(-v, fa, pc[r]);
            if (gr > j) y = fma_(gr == j + 1 ? -one_<T>() : -col1[r], fb, y);
            pc[r] = y;
          }
        }
        if (tid == 0 && j >= r0 && j < r0 + nr) col[j - r0] = beta;
        if (tid == 0 && jy >= 0 && jy < nr) col1[jy] = sc1[0];
        __syncthreads();
        j += 2;
      } else {
        for (int r = rs + tid; r < nr; r += blockDim.x) col[r] = col[r] * scal;
        __syncthreads();
        for (int c = j + 1 + wid; c < jb; c += nw) {
          const T f = wsh[c];
          T* pc = Ps + c * ldp;
          for (int r = rj + lane; r < nr; r += 32) {
            const T v = (r0 + r == j) ? one_<T>() : col[r];
            pc[r] = fma_(-v, f, pc[r]);
          }
        }
        if (tid == 0 && j >= r0 && j < r0 + nr) col[j - r0] = beta;
        __syncthreads();
        j += 1;
      }
      continue;
    }
    R xnorm = R(0);  // meaningful in thread 0 only (the scalars below)
    if (rescale) {
      // rare: rescale by 2^-e, e the exponent of the largest magnitude
      // (clamped so the scale itself stays finite), then sum again
      int e = 0;
      frexp(sc_r[1], &e);
      e = e > 1000 ? 1000 : (e < -1000 ? -1000 : e);
      const R scale = ldexp(R(1), -e);
      R ss2 = R(0);
      for (int r = rs + tid; r < nr; r += blockDim.x) ssq_scaled_add(ss2, col[r], scale);
      ss2 = block_sum(ss2, red_r);
      if (tid == 0) a.part_nrm[6 * a.gstride + b] = ss2;
      if (!panel_sync<SYNC>(a.bar, nsync, a.status, cflag)) return;
      if (wid == 0) {
        R s2 = R(0);
        for (int q = lane; q < G; q += 32) s2 += ld_cg(&a.part_nrm[6 * a.gstride + q]);
        s2 = warp_sum(s2);
        if (lane == 0) sc_r[2] = sqrt(s2) * ldexp(R(1), e);
      }
      __syncthreads();
      xnorm = sc_r[2];
    }
    if (tid == 0) {
      T beta, tau, scal;
      if (rescale) larfg_scalars(rowj[j], xnorm, beta, tau, scal);
      else larfg_scalars_ssq(rowj[j], sc_r[0], sc_r[1], beta, tau, scal);
      sc[0] = beta;
      sc[1] = tau;
      sc[2] = scal;
    }
    __syncthreads();
    const T beta = sc[0], tau = sc[1], scal = sc[2];
    if (b == 0 && tid == 0) a.tau[j] = tau;
    if (j + 1 >= jb) {
      for (int r = rs + tid; r < nr; r += blockDim.x) col[r] = col[r] * scal;
      if (tid == 0 && j >= r0 && j < r0 + nr) col[j - r0] = beta;
      __syncthreads();
      break;
    }
    if (!rescale) {
      // f_c = conj(tau) w_c, w_c = A[j, c] + conj(scal) d_c, formed once
      if (wid == 0) {
        T sum = zero_<T>();
        for (int w = 0; w < nw; w++) sum += red_w[w][lane];
        if (lane > j && lane < jb) wsh[lane] = conj_(tau) * fma_(conj_(scal), sum, rowj[lane]);
      }
    } else {
      // the two-round form on the scaled column: w = v^H A from v itself
      for (int r = rs + tid; r < nr; r += blockDim.x) col[r] = col[r] * scal;
      __syncthreads();
      const int rj = max(0, j - r0);
      T* pw2 = a.part_w + (int64_t)2 * a.gstride * NBMAX;
      for (int c = j + 1 + wid; c < jb; c += nw) {
        T s = zero_<T>();
        for (int r = rj + lane; r < nr; r += 32) {
          const T v = (r0 + r == j) ? one_<T>() : col[r];
          s = fma_(conj_(v), Ps[r + c * ldp], s);
        }
        s = warp_sum(s);
        if (lane == 0) pw2[(int64_t)b * NBMAX + c] = s;
      }
      if (!panel_sync<SYNC>(a.bar, nsync, a.status, cflag)) return;
      {
        const int per = (G + nw - 1) / nw;
        const int q0 = wid * per, q1 = min(G, q0 + per);
        T acc = zero_<T>();
        if (lane > j && lane < jb)
          for (int q = q0; q < q1; q++) acc += ld_cg(&pw2[(int64_t)q * NBMAX + lane]);
        red_w[wid][lane] = acc;
      }
      __syncthreads();
      if (wid == 0) {
        T sum = zero_<T>();
        for (int w = 0; w < nw; w++) sum += red_w[w][lane];
        if (lane > j && lane < jb) wsh[lane] = conj_(tau) * sum;
      }
    }
    __syncthreads();
    // ---- update rows >= j of the columns c > j: A[r, c] -= v_r f_c, with
    // v_j = 1 and v_r = scal x_r below (stored back as the reflector)
    // The reflector is scaled in place first; the update then gives each
    // warp its own columns (lanes over rows), so that all eight warps share
    // the FP64 work even when a CTA owns only a few dozen rows.
    const int rj = max(0, j - r0);
    if (!rescale)
      for (int r = rs + tid; r < nr; r += blockDim.x) col[r] = col[r] * scal;
    __syncthreads();
    for (int c = j + 1 + wid; c < jb; c += nw) {
      const T f = wsh[c];
      T* pc = Ps + c * ldp;
      for (int r = rj + lane; r < nr; r += 32) {
        const T v = (r0 + r == j) ? one_<T>() : col[r];
        pc[r] = fma_(-v, f, pc[r]);
      }
    }
    if (tid == 0 && j >= r0 && j < r0 + nr) col[j - r0] = beta;
    __syncthreads();
    j += 1;
  }

  // ---- Gram partials of V (unit lower trapezoidal) for the T factor: one
  // thread per pair (i, jj), i < jj, over this CTA's rows (no reductions)
  const int npairs = jb * (jb - 1) / 2;
  for (int pq = tid; pq < npairs; pq += blockDim.x) {
    int jj = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)pq)) * 0.5f);
    while (jj * (jj - 1) / 2 > pq) jj--;
    while (jj * (jj + 1) / 2 <= pq) jj++;
    const int i = pq - jj * (jj - 1) / 2;
    T s0 = zero_<T>(), s1 = zero_<T>();
    const int rb = max(0, jj - r0);
    int r = rb;
    if (r < nr && r0 + r == jj) {  // v_jj = 1 on its diagonal row
      s0 = conj_(Ps[r + i * ldp]);
      r++;
    }
    for (; r + 1 < nr; r += 2) {
      s0 = fma_(conj_(Ps[r + i * ldp]), Ps[r + jj * ldp], s0);
      s1 = fma_(conj_(Ps[r + 1 + i * ldp]), Ps[r + 1 + jj * ldp], s1);
    }
    if (r < nr) s0 = fma_(conj_(Ps[r + i * ldp]), Ps[r + jj * ldp], s0);
    a.part_g[(int64_t)b * NBMAX * NBMAX + i + jj * NBMAX] = s0 + s1;
  }
  for (int c = 0; c < jb; c++)
    for (int r = tid; r < nr; r += blockDim.x) a.A[(r0 + r) + (int64_t)c * a.lda] = Ps[r + c * ldp];
  if (!panel_sync<SYNC>(a.bar, nsync, a.status, cflag)) return;

  // ---- reduce the Gram over the CTAs: one thread per pair, the CTAs'
  // partials in a fixed order (four interleaved accumulators)
  for (int pq = b * (int)blockDim.x + tid; pq < npairs; pq += G * (int)blockDim.x) {
    int jj = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)pq)) * 0.5f);
    while (jj * (jj - 1) / 2 > pq) jj--;
    while (jj * (jj + 1) / 2 <= pq) jj++;
    const int i = pq - jj * (jj - 1) / 2;
    const T* src = a.part_g + i + jj * NBMAX;
    constexpr int64_t NN = NBMAX * NBMAX;
    T s0 = zero_<T>(), s1 = zero_<T>(), s2 = zero_<T>(), s3 = zero_<T>();
    int q = 0;
    for (; q + 3 < G; q += 4) {
      s0 += ld_cg(src + q * NN);
      s1 += ld_cg(src + (q + 1) * NN);
      s2 += ld_cg(src + (q + 2) * NN);
      s3 += ld_cg(src + (q + 3) * NN);
    }
    for (; q < G; q++) s0 += ld_cg(src + q * NN);
    a.gram[i + jj * NBMAX] = (s0 + s1) + (s2 + s3);
  }
  if (!panel_sync<SYNC>(a.bar, nsync, a.status, cflag)) return;

  // ---- T factor (larft, forward, column-wise): T = U^{-1} with U_ii =
  // 1/tau_i and U_il = G_il (i < l), each column an independent back
  // substitution x_k = tau_k, x_i = -tau_i sum_{l=i+1..k} G_il x_l (tau_i as
  // a factor: tau_i = 0 needs no division).  Column k goes to warp k mod 8
  // of CTA k / 8 (then every G * 8 columns); lane i owns row i.  tau and the
  // strict upper triangle of the Gram matrix are staged in shared memory
  // first (one batch of independent loads), so the substitution chain
  // itself waits on no L2 round trip.
  const int kfirst = b * nw;
  if (kfirst >= NBMAX) return;  // the same for every thread of the CTA
  __shared__ T gs[NBMAX * NBMAX];
  __shared__ T ts[NBMAX];
  if (kfirst < jb) {
    for (int e = tid; e < NBMAX * NBMAX; e += blockDim.x) {
      const int i = e % NBMAX, l = e / NBMAX;
      if (i < l && l < jb) gs[e] = ld_cg(&a.gram[e]);
    }
    if (tid < NBMAX) ts[tid] = tid < jb ? ld_cg(&a.tau[tid]) : zero_<T>();
  }
  __syncthreads();
  for (int k = kfirst + wid; k < NBMAX; k += G * nw) {
    T x = zero_<T>();
    if (k < jb) {
      T acc = zero_<T>();
      for (int l = k; l >= 0; l--) {
        const T mine = (l == k) ? ts[k] : -(ts[l] * acc);
        const T xl = shfl_idx_(mine, l);
        if (lane == l) x = xl;
        if (lane < l) acc = fma_(gs[lane + l * NBMAX], xl, acc);
      }
    }
    a.Tm[lane + k * NBMAX] = (k < jb && lane <= k) ? x : zero_<T>();
  }
}

// W2[:, c] = op(Tm) * sum_s Wpart[s][:, c]   (op = ^H for the factorization,
// identity for Q formation).  Fixed summation order -> deterministic.
template <class T>
__global__ void __launch_bounds__(256) reduce_trmm_kernel(int jb, int nt, int splits,
                                                          const T* __restrict__ Wpart,
                                                          int64_t sstride,
                                                          const T* __restrict__ Tm, int conjtrans,
                                                          T* __restrict__ W2) {
  __shared__ T Ts[NBMAX][NBMAX + 1];
  __shared__ T Ws[NBMAX][33];
  const int c0 = blockIdx.x * 32;
  for (int e = threadIdx.x; e < jb * jb; e += blockDim.x) {
    const int i = e % jb, l = e / jb;
    Ts[i][l] = conjtrans ? conj_(Tm[l + i * NBMAX]) : Tm[i + l * NBMAX];
  }
  for (int e = threadIdx.x; e < jb * 32; e += blockDim.x) {
    const int i = e % jb, cc = e / jb;
    T s = zero_<T>();
    if (c0 + cc < nt)
      for (int q = 0; q < splits; q++) s += Wpart[q * sstride + i + (int64_t)(c0 + cc) * jb];
    Ws[i][cc] = s;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < jb * 32; e += blockDim.x) {
    const int i = e % jb, cc = e / jb;
    if (c0 + cc >= nt) continue;
    T s = zero_<T>();
    for (int l = 0; l < jb; l++) s = fma_(Ts[i][l], Ws[l][cc], s);
    W2[i + (int64_t)(c0 + cc) * jb] = s;
  }
}

constexpr int QR_OUTER_NB = 128;  // outer block of the mixed-precision path
// SMs given to the look-ahead side stream (panels and the block Gram) while
// the main stream's persistent tensor-core grid takes the rest; 48 by
// default, MAK_LOOKAHEAD_CTAS overrides it (read once, clamped to 8..120).
int lookahead_ctas() { return (int)tuning(TUNE_LOOKAHEAD_CTAS); }
// In the tail of the factorization the far update shrinks below the time
// of the next block's panels; from MAK_LOOKAHEAD_TAIL_COLS far columns
// down, the side stream takes MAK_LOOKAHEAD_TAIL_CTAS SMs instead.
static int side_ctas(int64_t far_cols) {
  const double tail = tuning(TUNE_LOOKAHEAD_TAIL_COLS);
  return (double)far_cols <= tail ? (int)tuning(TUNE_LOOKAHEAD_TAIL_CTAS) : lookahead_ctas();
}
static thread_local int tl_side_ctas = 0;  // the side stream's SMs for the block being factored

static thread_local bool tl_no_lookahead = false;
bool lookahead_enabled() { return !tl_no_lookahead; }
void set_lookahead(bool on) { tl_no_lookahead = !on; }
static thread_local int tl_gemm_budget = 0;
int split_gemm_cta_budget() { return tl_gemm_budget; }
void set_split_gemm_cta_budget(int ctas) { tl_gemm_budget = ctas > 0 ? ctas : 0; }

// Side stream (highest priority, so its panel CTAs are scheduled ahead of
// the trailing GEMM's) and events of the look-ahead, one set per (host
// thread, device) so that calls from several threads never share an event
// and a call on another device never queues work on this device's stream;
// created by the first large call of that thread on that device (which must
// precede any graph capture there).
LookAhead* lookahead() {
  static thread_local LookAhead la[kMaxDevices];
  static thread_local int state[kMaxDevices] = {};  // 0 not created, 1 ready, -1 failed
  const int d = current_device();
  if (state[d] == 0) {
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    state[d] =
        (cudaStreamCreateWithPriority(&la[d].side, cudaStreamNonBlocking, hi) == cudaSuccess &&
         cudaEventCreateWithFlags(&la[d].ev_ready, cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&la[d].ev_done, cudaEventDisableTiming) == cudaSuccess)
            ? 1
            : -1;
  }
  return state[d] == 1 ? &la[d] : nullptr;
}

// T factor of a JB-wide block reflector (LAPACK larft, forward, column-wise
// storage: H_1 ... H_JB = I - V T V^H) from the Gram matrix G = V^H V and
// tau.  T is the inverse of the upper triangular U with U_ii = 1/tau_i and
// U_il = G_il (i < l): the larft recurrence T[0:j, j] = -tau_j T[0:j, 0:j]
// G[0:j, j], T[j, j] = tau_j, satisfies T U = I column by column.  Every
// column of T is therefore an independent back substitution,
//   x_k = tau_k,   x_i = -tau_i sum_{l=i+1..k} G_il x_l   (i < k),
// written with tau_i as a factor so that tau_i = 0 (an identity reflector)
// zeroes its row and column of T without a division.  One warp per column;
// lane t owns rows t, t + 32, t + 64, t + 96.
template <class T>
__global__ void __launch_bounds__(256) larft_cols_kernel(int jb, const T* __restrict__ G, int ldg,
                                                         const T* __restrict__ tau, T* Tout,
                                                         int ldt) {
  constexpr int RPL = QR_OUTER_NB / 32;
  const int lane = threadIdx.x & 31;
  const int k = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (k >= jb) return;
  T acc[RPL], x[RPL];
#pragma unroll
  for (int r = 0; r < RPL; r++) {
    acc[r] = zero_<T>();
    x[r] = zero_<T>();
  }
  for (int l = k; l >= 0; l--) {
    const int slot = l >> 5, owner = l & 31;
    T mine = acc[0];
#pragma unroll
    for (int r = 1; r < RPL; r++)
      if (slot == r) mine = acc[r];
    const T xl = (l == k) ? tau[k] : shfl_idx_(-(tau[l] * mine), owner);
#pragma unroll
    for (int r = 0; r < RPL; r++) {
      if (slot == r && lane == owner) x[r] = xl;
      const int i = lane + 32 * r;
      if (i < l) acc[r] = fma_(G[i + (int64_t)l * ldg], xl, acc[r]);
    }
  }
#pragma unroll
  for (int r = 0; r < RPL; r++) {
    const int i = lane + 32 * r;
    if (i < jb) Tout[i + (int64_t)k * ldt] = (i <= k) ? x[r] : zero_<T>();
  }
}

template <class T>
__global__ void signs_kernel(int k, const T* A, int64_t lda, int positive, T* s) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < k) s[j] = positive ? sign_safe_(A[j + j * lda]) : one_<T>();
}

// R[i, j] = (i <= j && i < k) ? conj(s_i) A[i, j] : 0   for i < rrows, j < n
template <class T>
__global__ void extract_r_kernel(int64_t rrows, int64_t n, int64_t k, const T* A, int64_t lda,
                                 const T* s, T* R, int64_t ldr) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t j = blockIdx.y;
  for (; j < n; j += gridDim.y) {
    if (i >= rrows) return;
    T v = zero_<T>();
    if (i <= j && i < k) v = conj_(s[i]) * A[i + j * lda];
    R[i + j * ldr] = v;
  }
}

// Q = [diag(s); 0] on the first k columns, identity beyond (qr_full)
template <class T>
__global__ void init_q_kernel(int64_t m, int64_t qcols, int64_t k, const T* s, T* Q, int64_t ldq) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int64_t j = blockIdx.y; j < qcols; j += gridDim.y) {
    if (i >= m) return;
    T v = zero_<T>();
    if (i == j) v = (j < k) ? s[j] : one_<T>();
    Q[i + j * ldq] = v;
  }
}

__global__ void info_reset_kernel(mak_info* info) {
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

int info_reset(cudaStream_t st, mak_info* info) {
  note_launch();
  info_reset_kernel<<<1, 1, 0, st>>>(info);
  return cudaGetLastError() == cudaSuccess ? 0 : MAK_ERR_CUDA;
}

std::atomic<unsigned long long>& launch_counter() {
  static std::atomic<unsigned long long> c{0};
  return c;
}

int num_sms() {
  static PerDevice<int> pd;
  return pd.get([] {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, current_device());
    return v > 0 ? v : 152;
  });
}
int max_smem_optin() {
  static PerDevice<int> pd;
  return pd.get([] {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, current_device());
    return v > 0 ? v : 227 * 1024;
  });
}

// Shared memory available to the panel slab: the opt-in maximum minus the
// kernel's static shared memory (T-factor scratch); queried, and the
// kernel's dynamic shared-memory limit raised, once per type and device.
template <class T>
static size_t panel_slab_cap() {
  static PerDevice<size_t> pd;
  return pd.get([] {
    cudaFuncAttributes fa;
    size_t stat = 48 * 1024;
    if (cudaFuncGetAttributes(&fa, qr_panel_kernel<T, SYNC_GRID>) == cudaSuccess)
      stat = fa.sharedSizeBytes;
    if (cudaFuncGetAttributes(&fa, qr_panel_kernel<T, SYNC_CLUSTER>) == cudaSuccess &&
        fa.sharedSizeBytes > stat)
      stat = fa.sharedSizeBytes;
    const size_t cap = (size_t)max_smem_optin() - stat - 1024;
    cudaFuncSetAttribute(qr_panel_kernel<T, SYNC_GRID>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap);
    cudaFuncSetAttribute(qr_panel_kernel<T, SYNC_CLUSTER>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap);
    cudaFuncSetAttribute(qr_panel_kernel<T, SYNC_HIER>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap);
    return cap;
  });
}

// Panels of at most this many rows per CTA (times the cluster limit) run as
// one thread-block cluster: below it a column's FP64 work per CTA stays
// smaller than what a global barrier costs.
constexpr int PANEL_CLUSTER_ROWS = 256;

// Launch shape of the panel kernel.  Cluster (sync = SYNC_CLUSTER): panels
// of up to kPanelClusterMax x PANEL_CLUSTER_ROWS rows, at least 64 rows per
// CTA.  Cooperative grid (SYNC_GRID) beyond that: rows per CTA bounded below
// by 64 (a grid barrier is only paid when there is real parallel work) and
// above by the shared-memory slab size; at most one CTA per SM.
struct PanelShape {
  int G, rpc, sync;
  int cl = 1;  // CTAs per cluster (SYNC_CLUSTER: G; SYNC_HIER: the cluster size)
  size_t smem;
};
template <class T>
static int panel_shape(int64_t mp, int jb, PanelShape& ps, int want_ctas) {
  const int max_ctas = num_sms();
  const size_t cap = panel_slab_cap<T>();
  int64_t rpc_max = (int64_t)(cap / ((size_t)jb * sizeof(T))) - 1;  // ld = rpc | 1
  const int64_t cl_rows = rpc_max < PANEL_CLUSTER_ROWS ? rpc_max : PANEL_CLUSTER_ROWS;
  if (mp <= (int64_t)kPanelClusterMax * cl_rows) {
    int64_t G = ceil_div(mp, 64);
    if (G > kPanelClusterMax) G = kPanelClusterMax;
    if (G < 1) G = 1;
    int64_t rpc = ceil_div(mp, G);
    if (rpc < 1) rpc = 1;
    G = ceil_div(mp, rpc);
    if (G < 1) G = 1;
    ps.G = (int)G;
    ps.rpc = (int)rpc;
    ps.sync = SYNC_CLUSTER;
    ps.cl = (int)G;
    ps.smem = (size_t)(ps.rpc | 1) * jb * sizeof(T);
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    cfg.gridDim = dim3((unsigned)G);
    cfg.blockDim = dim3(PANEL_THREADS);
    cfg.dynamicSmemBytes = ps.smem;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)G;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, qr_panel_kernel<T, SYNC_CLUSTER>, &cfg) ==
            cudaSuccess &&
        nclusters >= 1)
      return 0;
    (void)cudaGetLastError();  // fall through to the cooperative grid
  }
  // taller panels: a cooperative grid of clusters of C CTAs when the tuning
  // table asks for it (MAK_PANEL_HIER_C), else a plain cooperative grid
  const int hc = (int)tuning(TUNE_PANEL_HIER_C);
  if (hc == 2 || hc == 4 || hc == 8) {
    int64_t H = ceil_div(ceil_div(mp, 64), hc);
    if (H * hc > want_ctas) H = want_ctas / hc;
    if (H * hc > max_ctas) H = max_ctas / hc;
    if (H >= 1) {
      int64_t rpc = ceil_div(mp, H * hc);
      if (rpc <= rpc_max) {
        ps.G = (int)(H * hc);
        ps.rpc = (int)rpc;
        ps.sync = SYNC_HIER;
        ps.cl = hc;
        ps.smem = (size_t)(ps.rpc | 1) * jb * sizeof(T);
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute attr[1];
        cfg.gridDim = dim3((unsigned)ps.G);
        cfg.blockDim = dim3(PANEL_THREADS);
        cfg.dynamicSmemBytes = ps.smem;
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)hc;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, qr_panel_kernel<T, SYNC_HIER>, &cfg) ==
                cudaSuccess &&
            nclusters >= H)
          return 0;
        (void)cudaGetLastError();
      }
    }
  }
  int64_t G = ceil_div(mp, 64);
  if (G > want_ctas) G = want_ctas;
  if (G > max_ctas) G = max_ctas;
  if (G < 1) G = 1;
  int64_t rpc = ceil_div(mp, G);
  if (rpc > rpc_max) {
    G = ceil_div(mp, rpc_max);
    if (G > max_ctas) return MAK_ERR_UNSUPPORTED;
    rpc = ceil_div(mp, G);
  }
  if (rpc < 1) rpc = 1;
  G = ceil_div(mp, rpc);
  if (G < 1) G = 1;
  ps.G = (int)G;
  ps.rpc = (int)rpc;
  ps.sync = SYNC_GRID;
  ps.cl = 1;
  ps.smem = (size_t)(ps.rpc | 1) * jb * sizeof(T);
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, qr_panel_kernel<T, SYNC_GRID>,
                                                    PANEL_THREADS, ps.smem) != cudaSuccess)
    return MAK_ERR_CUDA;
  if ((int64_t)per_sm * max_ctas < G) return MAK_ERR_UNSUPPORTED;
  return 0;
}

template <class T>
int qr_run(cudaStream_t st, int64_t m, int64_t n, T* A, int64_t lda, T* Q, int64_t ldq,
           int64_t qcols, T* R, int64_t ldr, int64_t rrows, int positive, int blocksize,
           int precision, Arena& ar, mak_info* info) {
  const int64_t k = m < n ? m : n;
  const int nb = (blocksize > 0 && blocksize < NBMAX) ? blocksize : NBMAX;
  const int64_t nblk = ceil_div(k, nb);
  const int64_t wmax = (n > qcols ? n : qcols);
  const int sms = num_sms();
  const int gmax = sms;  // upper bound on panel CTAs (for workspace sizing)
  const int max_splits = 64;
  // mixed precision: 128-wide outer blocks whose block reflector is applied
  // with split-precision tensor-core GEMMs (K = 128 or K = m)
  // the 128-wide blocking pays only when its products are large enough to
  // take the split tensor-core path (gemm_prec's threshold); smaller
  // problems run the native blocking even when mixed precision is asked for
  const bool mixed = precision == MAK_PREC_MIXED && sizeof(real_t<T>) == 8 &&
                     (traits<T>::cpx ? 4.0 : 1.0) * (double)m * (double)n * QR_OUTER_NB >=
                         split_min_mnk();
  // outer block of the mixed path: 128 columns, or 64 for blocks whose
  // columns number at most MAK_QR_OUTER64_MAX_N (default 0: never), where
  // fewer 32-wide panels per block leave fewer within-block native updates
  const int NBO = mixed ? ((double)n <= tuning(TUNE_QR_OUTER64_MAX_N) ? 64 : QR_OUTER_NB) : nb;
  const int64_t nblk_o = ceil_div(k, NBO);

  T* tau = ar.take<T>(k > 0 ? k : 1);
  T* Ts = ar.take<T>((size_t)(nblk > 0 ? nblk : 1) * NBMAX * NBMAX);
  T* sgn = ar.take<T>(k > 0 ? k : 1);
  T* Wpart = ar.take<T>((size_t)max_splits * nb * (wmax > 0 ? wmax : 1));
  T* W2 = ar.take<T>((size_t)nb * (wmax > 0 ? wmax : 1));
  // norm partials [2 round parities][3][gmax] + the rescaled sums [gmax];
  // dot partials [2 parities][gmax][NBMAX] + the rescaled path's [gmax][NBMAX]
  // + column j+1's [2 parities][gmax][NBMAX]
  real_t<T>* part_nrm = ar.take<real_t<T>>((size_t)7 * gmax);
  T* part_w = ar.take<T>((size_t)5 * gmax * NBMAX);
  T* part_g = ar.take<T>((size_t)gmax * NBMAX * NBMAX);
  T* alpha_buf = ar.take<T>(4 * NBMAX);  // rows j and j+1 of the panel, by round parity
  T* gram_buf = ar.take<T>((size_t)NBMAX * NBMAX);
  unsigned* bar = ar.take<unsigned>(2);
  int* cflag = ar.take<int>(gmax);
  T *To = nullptr, *Gm = nullptr, *Wm = nullptr, *W2m = nullptr;
  char* ozs = nullptr;
  size_t oz_bytes = 0;
  if (mixed) {
    To = ar.take<T>((size_t)(nblk_o > 0 ? nblk_o : 1) * NBO * NBO);
    Gm = ar.take<T>((size_t)NBO * NBO);
    Wm = ar.take<T>((size_t)NBO * (wmax > 0 ? wmax : 1));
    W2m = ar.take<T>((size_t)NBO * (wmax > 0 ? wmax : 1));
    // the tensor-core GEMMs run one after another and share one scratch region
    const int64_t shapes[4][3] = {{NBO, wmax, m}, {m, wmax, NBO}, {NBO, wmax, NBO}, {NBO, NBO, m}};
    for (auto& sh : shapes) {
      Arena meas(nullptr, 0);
      gemm_prec<T>(st, precision, sh[0], sh[1], sh[2], one_<T>(), opnd<T>(nullptr, 1),
                   opnd<T>(nullptr, 1), zero_<T>(), nullptr, 1, meas, nullptr);
      if (meas.off + 1024 > oz_bytes) oz_bytes = meas.off + 1024;
    }
    ozs = ar.take<char>(oz_bytes);
  }
  // the block Gram matrix and the within-block updates of the panels run on
  // the look-ahead stream: their own scratch, and (mixed) W / T^H W of a
  // panel's update
  size_t gram_bytes = 0;
  char* grams = nullptr;
  T *Wp = nullptr, *W2p = nullptr;
  const bool panel_split = mixed && tuning(TUNE_QR_PANEL_SPLIT) != 0;
  if (mixed) {
    const int64_t shapes[3][3] = {{NBO, NBO, m}, {NBMAX, NBO, m}, {m, NBO, NBMAX}};
    for (int q = 0; q < (panel_split ? 3 : 1); q++) {
      Arena meas(nullptr, 0);
      gemm_prec<T>(st, precision, shapes[q][0], shapes[q][1], shapes[q][2], one_<T>(),
                   opnd<T>(nullptr, 1), opnd<T>(nullptr, 1), zero_<T>(), nullptr, 1, meas,
                   nullptr);
      if (meas.off + 1024 > gram_bytes) gram_bytes = meas.off + 1024;
    }
    grams = ar.take<char>(gram_bytes);
    if (panel_split) {
      Wp = ar.take<T>((size_t)NBMAX * NBO);
      W2p = ar.take<T>((size_t)NBMAX * NBO);
    }
  }
  if (ar.base == nullptr) return 0;
  if (!ar.ok()) return MAK_ERR_WORKSPACE;
  int* status = &info->status;

  MAK_CUDA_TRY(cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), st));

  // C <- (I - V op(T) V^H) C with the tensor-core GEMMs; op(T) = T^H for the
  // factorization, T for Q formation (T is JB x JB upper, ld NBO)
  // max_ctas > 0 leaves the other SMs to the look-ahead side stream
  auto larfb_mixed = [&](const T* V, int64_t mp, int JB, const T* Tm, int conjtrans, T* Cm,
                         int64_t ldc, int64_t nc, cudaStream_t s, int max_ctas) -> int {
    if (nc <= 0) return 0;
    {
      Arena oz(ozs, oz_bytes);
      MAK_TRY(gemm_prec<T>(s, precision, JB, nc, mp, one_<T>(),
                           opnd<T>(V, lda, OP_C, MASK_UNIT_LOWER), opnd<T>(Cm, ldc), zero_<T>(),
                           Wm, JB, oz, status, max_ctas));
    }
    {
      Arena oz(ozs, oz_bytes);
      MAK_TRY(gemm_prec<T>(s, precision, JB, nc, JB, one_<T>(),
                           opnd<T>(Tm, NBO, conjtrans ? OP_C : OP_N, MASK_UPPER),
                           opnd<T>(Wm, JB), zero_<T>(), W2m, JB, oz, status, max_ctas));
    }
    Arena oz(ozs, oz_bytes);
    return gemm_prec<T>(s, precision, mp, nc, JB, -one_<T>(),
                        opnd<T>(V, lda, OP_N, MASK_UNIT_LOWER), opnd<T>(W2m, JB), one_<T>(), Cm,
                        ldc, oz, status, max_ctas);
  };
  // C = A[j0:, c0:c1] <- (I - V T^H V^H)... with the native SIMT kernels
  auto larfb_native = [&](int64_t j0, int jb, const T* Tb, int64_t c0, int64_t c1,
                          cudaStream_t s) -> int {
    const int64_t nt = c1 - c0;
    if (nt <= 0) return 0;
    const int64_t mp = m - j0;
    const T* Ap = A + j0 + j0 * lda;
    T* C = A + j0 + c0 * lda;
    int splits = pick_splits(jb, nt, mp, sms);
    if (splits > max_splits) splits = max_splits;
    int used = 1;
    MAK_TRY(gemm<T>(s, jb, nt, mp, one_<T>(), opnd<T>(Ap, lda, OP_C, MASK_UNIT_LOWER),
                    opnd<T>(C, lda), zero_<T>(), Wpart, jb, splits, (int64_t)jb * nt, &used));
    note_launch();
    reduce_trmm_kernel<T><<<(unsigned)ceil_div(nt, 32), 256, 0, s>>>(jb, (int)nt, used, Wpart,
                                                                      (int64_t)jb * nt, Tb, 1, W2);
    MAK_CUDA_TRY(cudaGetLastError());
    return gemm<T>(s, mp, nt, jb, -one_<T>(), opnd<T>(Ap, lda, OP_N, MASK_UNIT_LOWER),
                   opnd<T>(W2, jb), one_<T>(), C, lda);
  };
  // mixed: a 32-wide panel's reflector applied to the rest of its 128-wide
  // block with split products (W = V^H C, W2 = T^H W, C -= V W2) on the
  // side stream's scratch; gemm_prec keeps products below the split gate
  // native
  auto larfb_panel_split = [&](int64_t j0, int jb, const T* Tb, int64_t c0, int64_t c1,
                               cudaStream_t s) -> int {
    const int64_t nt = c1 - c0;
    if (nt <= 0) return 0;
    const int64_t mp = m - j0;
    const T* Ap = A + j0 + j0 * lda;
    T* C = A + j0 + c0 * lda;
    const int mc = s == st ? 0 : tl_side_ctas;
    {
      Arena ga(grams, gram_bytes);
      MAK_TRY(gemm_prec<T>(s, precision, jb, nt, mp, one_<T>(),
                           opnd<T>(Ap, lda, OP_C, MASK_UNIT_LOWER), opnd<T>(C, lda), zero_<T>(),
                           Wp, jb, ga, status, mc));
    }
    note_launch();
    reduce_trmm_kernel<T><<<(unsigned)ceil_div(nt, 32), 256, 0, s>>>(jb, (int)nt, 1, Wp,
                                                                      (int64_t)jb * nt, Tb, 1, W2p);
    MAK_CUDA_TRY(cudaGetLastError());
    Arena ga(grams, gram_bytes);
    return gemm_prec<T>(s, precision, mp, nt, jb, -one_<T>(),
                        opnd<T>(Ap, lda, OP_N, MASK_UNIT_LOWER), opnd<T>(W2p, jb), one_<T>(), C,
                        lda, ga, status, mc);
  };
  // one 32-wide panel (cooperative launch)
  // on the look-ahead stream the panel takes a few SMs only, leaving the
  // rest to the trailing GEMM it overlaps with
  auto panel = [&](int64_t j0, int jb, cudaStream_t s) -> int {
    const int64_t mp = m - j0;
    PanelShape ps;
    MAK_TRY(panel_shape<T>(mp, jb, ps, s == st ? sms : tl_side_ctas));
    PanelArgs<T> pa{A + j0 + j0 * lda, lda, (int)mp, jb, ps.rpc, tau + j0,
                    Ts + (j0 / nb) * NBMAX * NBMAX, part_nrm, part_w, part_g, alpha_buf,
                    gram_buf, bar, cflag, status, gmax, ps.sync != SYNC_HIER && tuning(TUNE_PANEL_PAIR) != 0};
    ProfScope prof(s, PROF_QR_PANEL, 2.0 * (double)mp * jb * sizeof(T));
    note_launch();
    if (ps.sync == SYNC_CLUSTER || ps.sync == SYNC_HIER) {
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute attr[2];
      cfg.gridDim = dim3((unsigned)ps.G);
      cfg.blockDim = dim3(PANEL_THREADS);
      cfg.dynamicSmemBytes = ps.smem;
      cfg.stream = s;
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = (unsigned)ps.cl;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      attr[1].id = cudaLaunchAttributeCooperative;
      attr[1].val.cooperative = 1;
      cfg.attrs = attr;
      cfg.numAttrs = ps.sync == SYNC_HIER ? 2 : 1;
      if (ps.sync == SYNC_HIER)
        MAK_CUDA_TRY(cudaLaunchKernelEx(&cfg, qr_panel_kernel<T, SYNC_HIER>, pa));
      else
        MAK_CUDA_TRY(cudaLaunchKernelEx(&cfg, qr_panel_kernel<T, SYNC_CLUSTER>, pa));
      return 0;
    }
    void* args[] = {&pa};
    MAK_CUDA_TRY(cudaLaunchCooperativeKernel((void*)qr_panel_kernel<T, SYNC_GRID>, dim3(ps.G),
                                             dim3(PANEL_THREADS), args, ps.smem, s));
    return 0;
  };
  // factor outer block b: its panels with updates confined to the block,
  // and (mixed) the 128-wide T factor from the block's Gram matrix
  auto factor_block = [&](int64_t b, cudaStream_t s) -> int {
    const int64_t J0 = b * NBO;
    const int JB = (int)((k - J0) < NBO ? (k - J0) : NBO);
    for (int64_t j0 = J0; j0 < J0 + JB; j0 += nb) {
      const int jb = (int)((J0 + JB - j0) < nb ? (J0 + JB - j0) : nb);
      MAK_TRY(panel(j0, jb, s));
      if (panel_split)
        MAK_TRY(larfb_panel_split(j0, jb, Ts + (j0 / nb) * NBMAX * NBMAX, j0 + jb, J0 + JB, s));
      else
        MAK_TRY(larfb_native(j0, jb, Ts + (j0 / nb) * NBMAX * NBMAX, j0 + jb, J0 + JB, s));
    }
    if (!mixed) return 0;
    const T* V = A + J0 + J0 * lda;
    {
      // the Gram matrix fixes the orthogonality of the block reflector; the
      // split-precision product is FP64-accurate, and 2 m 128^2 flops per
      // block on the FP64 pipe would sit on the look-ahead's critical path
      Arena ga(grams, gram_bytes);
      MAK_TRY(gemm_prec<T>(s, precision, JB, JB, m - J0, one_<T>(),
                           opnd<T>(V, lda, OP_C, MASK_UNIT_LOWER),
                           opnd<T>(V, lda, OP_N, MASK_UNIT_LOWER), zero_<T>(), Gm, NBO, ga,
                           status, s == st ? 0 : tl_side_ctas));
    }
    note_launch();
    larft_cols_kernel<T><<<(unsigned)ceil_div(JB, 8), 256, 0, s>>>(JB, Gm, NBO, tau + J0,
                                                                  To + b * NBO * NBO, NBO);
    MAK_CUDA_TRY(cudaGetLastError());
    return 0;
  };
  // block b's reflector applied to the columns [c0, c1)
  auto apply_block = [&](int64_t b, int64_t c0, int64_t c1, cudaStream_t s,
                         int max_ctas) -> int {
    const int64_t J0 = b * NBO;
    const int JB = (int)((k - J0) < NBO ? (k - J0) : NBO);
    if (mixed)
      return larfb_mixed(A + J0 + J0 * lda, m - J0, JB, To + b * NBO * NBO, 1,
                         A + J0 + c0 * lda, lda, c1 - c0, s, max_ctas);
    return larfb_native(J0, JB, Ts + (J0 / nb) * NBMAX * NBMAX, c0, c1, s);
  };

  // ------------------------------------------------------------ factor
  // Look-ahead: block b's reflector is applied first to block b+1's columns;
  // a high-priority side stream then factors block b+1 while the main stream
  // applies block b to the remaining columns, so the latency-bound panels
  // hide behind the large trailing GEMMs.
  LookAhead* la = (nblk_o > 1 && lookahead_enabled() && (double)m * n >= 4.0e6) ? lookahead()
                                                                                  : nullptr;
  if (nblk_o > 0) MAK_TRY(factor_block(0, st));
  for (int64_t b = 0; b < nblk_o; b++) {
    const int64_t J0 = b * NBO;
    const int64_t nx = J0 + ((k - J0) < NBO ? (k - J0) : NBO);          // first column of b+1
    const bool has_next = b + 1 < nblk_o;
    const int64_t nx_end = has_next ? nx + ((k - nx) < NBO ? (k - nx) : NBO) : nx;
    if (has_next && la) {
      MAK_TRY(apply_block(b, nx, nx_end, st, 0));
      MAK_CUDA_TRY(cudaEventRecord(la->ev_ready, st));
      MAK_CUDA_TRY(cudaStreamWaitEvent(la->side, la->ev_ready, 0));
      tl_side_ctas = side_ctas(n - nx_end);
      if (tl_side_ctas > sms - 8) tl_side_ctas = sms - 8;
      MAK_TRY(factor_block(b + 1, la->side));
      MAK_CUDA_TRY(cudaEventRecord(la->ev_done, la->side));
      // the persistent tensor-core grid leaves the side stream its SMs
      MAK_TRY(apply_block(b, nx_end, n, st, sms - tl_side_ctas));
      MAK_CUDA_TRY(cudaStreamWaitEvent(st, la->ev_done, 0));
    } else {
      MAK_TRY(apply_block(b, nx, n, st, 0));
      if (has_next) MAK_TRY(factor_block(b + 1, st));
    }
  }

  // ------------------------------------------------------ R and the gauge
  if (k > 0) {
    note_launch();
    signs_kernel<T><<<(unsigned)ceil_div(k, 256), 256, 0, st>>>((int)k, A, lda, positive, sgn);
    MAK_CUDA_TRY(cudaGetLastError());
  }
  if (R != nullptr && rrows > 0 && n > 0) {
    dim3 g((unsigned)ceil_div(rrows, 256), (unsigned)(n < 65535 ? n : 65535));
    note_launch();
    extract_r_kernel<T><<<g, 256, 0, st>>>(rrows, n, k, A, lda, sgn, R, ldr);
    MAK_CUDA_TRY(cudaGetLastError());
  }
  if (m > 0 && qcols > 0) {
    dim3 g((unsigned)ceil_div(m, 256), (unsigned)(qcols < 65535 ? qcols : 65535));
    note_launch();
    init_q_kernel<T><<<g, 256, 0, st>>>(m, qcols, k, sgn, Q, ldq);
    MAK_CUDA_TRY(cudaGetLastError());
  }

  // ------------------------------------------- Q = H_1 ... H_k [diag(s); 0]
  if (mixed) {
    for (int64_t bo = nblk_o - 1; bo >= 0; bo--) {
      const int64_t J0 = bo * NBO;
      const int JB = (int)((k - J0) < NBO ? (k - J0) : NBO);
      const int64_t qt = qcols - J0;
      if (qt <= 0) continue;
      MAK_TRY(larfb_mixed(A + J0 + J0 * lda, m - J0, JB, To + bo * NBO * NBO, 0,
                          Q + J0 + J0 * ldq, ldq, qt, st, 0));
    }
    return 0;
  }
  for (int64_t bi = nblk - 1; bi >= 0; bi--) {
    const int64_t j0 = bi * nb;
    const int jb = (int)((k - j0) < nb ? (k - j0) : nb);
    const int64_t mp = m - j0;
    const int64_t qt = qcols - j0;
    if (qt <= 0) continue;
    const T* Ap = A + j0 + j0 * lda;
    const T* Tb = Ts + bi * NBMAX * NBMAX;
    T* Qs = Q + j0 + j0 * ldq;
    int splits = pick_splits(jb, qt, mp, sms);
    if (splits > max_splits) splits = max_splits;
    int used = 1;
    MAK_TRY(gemm<T>(st, jb, qt, mp, one_<T>(), opnd<T>(Ap, lda, OP_C, MASK_UNIT_LOWER),
                    opnd<T>(Qs, ldq), zero_<T>(), Wpart, jb, splits, (int64_t)jb * qt, &used));
    note_launch();
    reduce_trmm_kernel<T><<<(unsigned)ceil_div(qt, 32), 256, 0, st>>>(
        jb, (int)qt, used, Wpart, (int64_t)jb * qt, Tb, 0, W2);
    MAK_CUDA_TRY(cudaGetLastError());
    MAK_TRY(gemm<T>(st, mp, qt, jb, -one_<T>(), opnd<T>(Ap, lda, OP_N, MASK_UNIT_LOWER),
                    opnd<T>(W2, jb), one_<T>(), Qs, ldq));
  }
  return 0;
}

#define MAK_INST_QR(T)                                                                        \
  template int qr_run<T>(cudaStream_t, int64_t, int64_t, T*, int64_t, T*, int64_t, int64_t, \
                         T*, int64_t, int64_t, int, int, int, Arena&, mak_info*);
MAK_INST_QR(double)
MAK_INST_QR(float)
MAK_INST_QR(zcomplex)
MAK_INST_QR(ccomplex)

// ------------------------------------------------------------ C entry ---

template <class T>
static int qr_entry(int full, int64_t m, int64_t n, void* Av, int64_t lda, void* Qv, int64_t ldq,
                    void* Rv, int64_t ldr, const mak_qr_opts* opts, void* work, size_t work_bytes,
                    mak_info* info, mak_stream_t stream) {
  T* A = (T*)Av;
  T* Q = (T*)Qv;
  T* R = (T*)Rv;
  if (m < 0) return -1;
  if (n < 0) return -2;
  const int64_t k = m < n ? m : n;
  const int64_t qcols = full ? m : k;
  const int64_t rrows = full ? m : k;
  if (A == nullptr && m * n > 0) return -3;
  if (lda < (m > 1 ? m : 1)) return -4;
  if (Q == nullptr && m * qcols > 0) return -5;
  if (Q != nullptr && (void*)Q == (void*)A) return -5;  // in-place Q is not provided
  if (ldq < (m > 1 ? m : 1)) return -6;
  if (R != nullptr && ldr < (rrows > 1 ? rrows : 1)) return -8;
  mak_qr_opts o{1, 0, MAK_PREC_NATIVE, 0};
  if (opts) o = *opts;
  if (o.blocksize < 0 || o.blocksize > NBMAX) return -9;
  if (o.precision != MAK_PREC_NATIVE && o.precision != MAK_PREC_MIXED) return -9;
  cudaStream_t st = (cudaStream_t)stream;
  Arena ar(work, work_bytes);
  mak_info* inf = info ? info : ar.take<mak_info>(1);
  if (work == nullptr && info == nullptr) return -11;
  // size check first (a measuring pass)
  {
    Arena meas(nullptr, 0);
    if (!info) meas.take<mak_info>(1);
    qr_run<T>(st, m, n, nullptr, lda, nullptr, ldq, qcols, nullptr, ldr, rrows, o.positive,
              o.blocksize, o.precision, meas, nullptr);
    if (meas.off > work_bytes) return -12;
  }
  MAK_TRY(info_reset(st, inf));
  return qr_run<T>(st, m, n, A, lda, Q, ldq, qcols, R, ldr, rrows, o.positive, o.blocksize,
                   o.precision, ar, inf);
}

}  // namespace mak

using namespace mak;

extern "C" {

int mak_qr_workspace(int dtype, int64_t m, int64_t n, int full, const mak_qr_opts* opts,
                     size_t* bytes) {
  if (bytes == nullptr) return -6;
  if (m < 0) return -2;
  if (n < 0) return -3;
  mak_qr_opts o{1, 0, MAK_PREC_NATIVE, 0};
  if (opts) o = *opts;
  const int64_t k = m < n ? m : n;
  const int64_t qcols = full ? m : k;
  const int64_t rrows = full ? m : k;
  Arena meas(nullptr, 0);
  meas.take<mak_info>(1);
  switch (dtype) {
    case MAK_F64: qr_run<double>(0, m, n, nullptr, m, nullptr, m, qcols, nullptr, rrows, rrows, o.positive, o.blocksize, o.precision, meas, nullptr); break;
    case MAK_C64: qr_run<zcomplex>(0, m, n, nullptr, m, nullptr, m, qcols, nullptr, rrows, rrows, o.positive, o.blocksize, o.precision, meas, nullptr); break;
    case MAK_F32: qr_run<float>(0, m, n, nullptr, m, nullptr, m, qcols, nullptr, rrows, rrows, o.positive, o.blocksize, o.precision, meas, nullptr); break;
    case MAK_C32: qr_run<ccomplex>(0, m, n, nullptr, m, nullptr, m, qcols, nullptr, rrows, rrows, o.positive, o.blocksize, o.precision, meas, nullptr); break;
    default: return -1;
  }
  *bytes = meas.off + 256;
  return 0;
}

#define MAK_QR_ENTRY(NAME, FULL, T, PT)                                                        \
  int NAME(int64_t m, int64_t n, PT* A, int64_t lda, PT* Q, int64_t ldq, PT* R, int64_t ldr,   \
           const mak_qr_opts* opts, void* work, size_t work_bytes, mak_info* info,             \
           mak_stream_t stream) {                                                              \
    return qr_entry<T>(FULL, m, n, A, lda, Q, ldq, R, ldr, opts, work, work_bytes, info,       \
                       stream);                                                                \
  }
MAK_QR_ENTRY(mak_qr_compact_d, 0, double, double)
MAK_QR_ENTRY(mak_qr_compact_z, 0, zcomplex, void)
MAK_QR_ENTRY(mak_qr_compact_s, 0, float, float)
MAK_QR_ENTRY(mak_qr_compact_c, 0, ccomplex, void)
MAK_QR_ENTRY(mak_qr_full_d, 1, double, double)
MAK_QR_ENTRY(mak_qr_full_z, 1, zcomplex, void)
MAK_QR_ENTRY(mak_qr_full_s, 1, float, float)
MAK_QR_ENTRY(mak_qr_full_c, 1, ccomplex, void)

uint64_t mak_kernel_launches(void) { return (uint64_t)launch_counter().load(); }

const char* mak_version(void) { return "mak_gb300 0.1.0 (sm_103a)"; }

const char* mak_status_string(int code) {
  if (code == MAK_OK) return "ok";
  if (code < 0) return "invalid argument (-index of the offending argument)";
  switch (code) {
    case MAK_ERR_CUDA: return "CUDA launch or runtime error";
    case MAK_ERR_TIMEOUT: return "bounded device-side wait gave up";
    case MAK_ERR_UNSUPPORTED: return "shape outside the supported envelope";
    case MAK_ERR_WORKSPACE: return "workspace too small";
    default: return "unknown status";
  }
}

}  // extern "C"
