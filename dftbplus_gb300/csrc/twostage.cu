// Two-stage tridiagonal reduction and back-transformation (see twostage.cuh for the scheme).
//
// Algorithm references (published methods, restated here): the band reduction with blocked
// two-sided updates W = A22 V T - 1/2 V (T^T V^T A22 V T), A22 -= W V^T + V W^T is the SBR
// dsytrd_sy2sb form (Bischof, Lang, Sun 2000); the bulge chasing with one reflector per band
// block and pipelined sweeps follows Haidar, Ltaief, Dongarra (SC'11) ("sb2st" kernels of type 1,
// 2, 3); the grouping of reflectors of consecutive sweeps into diamond/parallelogram WY blocks for
// the back-transformation follows the same work. Which reference call this replaces: the sytrd
// part of hegvd / magmaHegvd (math/eigensolver.F90:561-660, :1143-1245).
#include <algorithm>
#include <cmath>

#include "twostage.cuh"

namespace dg {

std::atomic<int> g_twostage{2};

namespace {

constexpr int kQrThreads = 256;
constexpr unsigned kChaseSpinLimit = 1u << 24;   // polls of a progress word before giving up (seconds)
constexpr int kSweepDone = 1 << 30;
constexpr int kL2 = kBand + kQ2Group - 1;         // rows of a stage-2 WY block

// Four consecutive elements of a 16-byte aligned shared array.
__device__ __forceinline__ void ld4(const float *p, float (&o)[4]) {
  const float4 v = *reinterpret_cast<const float4 *>(p);
  o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
}
__device__ __forceinline__ void ld4(const double *p, double (&o)[4]) {
  const double2 a = *reinterpret_cast<const double2 *>(p);
  const double2 b = *reinterpret_cast<const double2 *>(p + 2);
  o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
}


// --------------------------------------------------------------------------------- panel QR
// Householder QR of the m x nb panel P (column-major, ldp) with nb <= kBand, kr = min(m, nb)
// reflectors (LAPACK dgeqr2 semantics: beta = -sign(alpha) ||x||, tau = (beta - alpha) / beta,
// v = [1; x_tail / (alpha - beta)]). The rows are split over the CTAs of one cooperative launch
// (R >= nb rows each, so the top rows 0..kr-1 all live in CTA 0) and stay in shared memory for the
// whole panel. Column j needs one grid barrier: before it every CTA publishes, for its rows below
// j, the dots of column j with every column c >= j (x^T a_c); after it every CTA forms the same
// reflector from the summed dots and applies it to its own rows (w_c = v^T a_c = a_c[j] + scale
// * x_tail^T a_c_tail), then publishes the dots of column j + 1. Partial sums are added in a fixed
// order, so the result is deterministic.
// Output: V (m x nb, ldv): 0 above row c, 1 at row c, v below (zero columns for c >= kr);
// P: R (upper trapezoid), zeros below; tau[kr].
template <typename T>
struct PanelQrArgs {
  T *P;
  int ldp;
  T *V;
  int ldv;
  T *tau;
  int m, nb, kr, R;
  T *part;   // [2][G][nb] partial dots
  T *top;    // [2][nb] row j of the panel (CTA 0)
  GridBar *bar;
  int *status;
};

template <typename T>
__global__ void __launch_bounds__(kQrThreads) panel_qr_kernel(PanelQrArgs<T> a) {
  extern __shared__ __align__(16) unsigned char qr_smem[];
  T *sh = reinterpret_cast<T *>(qr_smem);   // [nb][R], column-major local panel
  __shared__ T sS[kBand], sTop[kBand], sW[kBand];
  __shared__ T sScal[3];
  const int G = gridDim.x, cta = blockIdx.x, t = threadIdx.x;
  const int R = a.R, nb = a.nb;
  const int r0 = cta * R, nr = max(0, min(a.m, r0 + R) - r0);
  const int warp = t >> 5, lane = t & 31;
  constexpr int NW = kQrThreads / 32;
  unsigned epoch = 0;
  for (int idx = t; idx < nb * R; idx += kQrThreads) {
    const int c = idx / R, i = idx - c * R;
    sh[idx] = (i < nr) ? a.P[(size_t)(r0 + i) + (size_t)c * a.ldp] : T(0);
  }
  __syncthreads();
  // dots of column jn with the columns c >= jn over this CTA's rows below jn, and row jn itself
  auto publish = [&](int jn, int buf) {
    for (int c = jn + warp; c < nb; c += NW) {
      T acc = T(0);
      for (int i = lane; i < nr; i += 32)
        if (r0 + i > jn) acc = fma(sh[jn * R + i], sh[c * R + i], acc);
      acc = warp_sum(acc);
      if (lane == 0) a.part[((size_t)buf * G + cta) * nb + c] = acc;
    }
    if (cta == 0)
      for (int c = jn + t; c < nb; c += kQrThreads) a.top[buf * nb + c] = sh[c * R + jn];
  };
  publish(0, 0);
  grid_sync(a.bar, (unsigned)G, epoch);
  for (int j = 0; j < a.kr; ++j) {
    const int buf = j & 1;
    for (int c = j + warp; c < nb; c += NW) {
      T acc = T(0);
      for (int q = lane; q < G; q += 32) acc += __ldcg(a.part + ((size_t)buf * G + q) * nb + c);
      acc = warp_sum(acc);
      if (lane == 0) {
        sS[c] = acc;
        sTop[c] = __ldcg(a.top + buf * nb + c);
      }
    }
    __syncthreads();
    if (t == 0) {
      const T alpha = sTop[j], ss = sS[j];
      T beta, tv, scale;
      if (ss == T(0)) {
        tv = T(0);
        beta = alpha;
        scale = T(0);
      } else {
        beta = -copysign(sqrt(alpha * alpha + ss), alpha);
        tv = (beta - alpha) / beta;
        scale = T(1) / (alpha - beta);
      }
      sScal[0] = tv;
      sScal[1] = scale;
      sScal[2] = beta;
      if (cta == 0) a.tau[j] = tv;
    }
    __syncthreads();
    const T tv = sScal[0], scale = sScal[1], beta = sScal[2];
    for (int c = j + 1 + t; c < nb; c += kQrThreads) sW[c] = tv * (sTop[c] + scale * sS[c]);   // tau w_c
    __syncthreads();
    // a_c -= tau w_c v for c > j (row j: v = 1; rows below: v = x scale)
    const int ncols = nb - j - 1;
    for (int idx = t; idx < ncols * R; idx += kQrThreads) {
      const int c = j + 1 + idx / R, i = idx % R;
      const int gi = r0 + i;
      if (i < nr && gi >= j) {
        const T f = sW[c];
        sh[c * R + i] -= (gi == j) ? f : f * scale * sh[j * R + i];
      }
    }
    __syncthreads();
    for (int i = t; i < nr; i += kQrThreads) {
      const int gi = r0 + i;
      if (gi == j) sh[j * R + i] = beta;
      else if (gi > j) sh[j * R + i] *= scale;
    }
    __syncthreads();
    if (j + 1 < a.kr) {
      publish(j + 1, buf ^ 1);
      grid_sync(a.bar, (unsigned)G, epoch);
    }
  }
  for (int idx = t; idx < nb * R; idx += kQrThreads) {
    const int c = idx / R, i = idx - c * R;
    if (i >= nr) continue;
    const int gi = r0 + i;
    const T val = sh[idx];
    const T vv = (c < a.kr) ? ((gi < c) ? T(0) : ((gi == c) ? T(1) : val)) : T(0);
    a.V[(size_t)gi + (size_t)c * a.ldv] = vv;
    a.P[(size_t)gi + (size_t)c * a.ldp] = (gi <= c) ? val : T(0);
  }
  if (t == 0 && a.status != nullptr && *(volatile int *)&a.bar->err != 0) atomicMax(a.status, (int)kDevIterCap);
}

// --------------------------------------------------------------------------------- bulge chasing
// Sweep s eliminates column s below the subdiagonal and chases the fill down the band:
//   task 0: reflector H_0 from A(s+1 : s+b, s) (e[s] = beta, d[s] = A(s,s)); D_0 <- H_0 D_0 H_0 with
//           D_0 = A(s+1 : s+b, s+1 : s+b);
//   task k >= 1 (c_k = s + 1 + k b): B_k = A(c_k : c_k+b-1, c_{k-1} : c_{k-1}+b-1) <- B_k H_{k-1};
//           reflector H_k from the first column of B_k (annihilates it below its top); the other
//           columns of B_k <- H_k B_k; D_k = A(c_k : c_k+b-1, c_k : c_k+b-1) <- H_k D_k H_k.
// Task k of sweep s touches rows/columns in [c_{k-1}, c_k + b - 1]; task k + 2 of sweep s - 1 starts
// at row c_k + b, so task k may run once sweep s - 1 has completed task k + 1 (progress >= k + 2).
// Only the lower triangle of A is read or written. One CTA works on one sweep at a time, sweeps
// are dealt round-robin over the co-resident CTAs of a cooperative launch, so the chain of waits
// always ends at a running sweep. Every wait is bounded.
template <typename T>
struct ChaseArgs {
  T *A;
  int lda, n, kmax;
  T *d, *e;
  T *V2, *tau2;      // stage-2 WY blocks (kL2 x kQ2Group each, row-major) and their tau
  int *progress;     // [n]: tasks completed per sweep (kSweepDone when finished)
  int *err;
  int *status;
};

// Progress words: a release store after the warp's (or CTA's) writes of a task, an acquire load
// before the dependent task reads them. The writers' stores are ordered before the releasing lane's
// store by the preceding __syncwarp/__syncthreads; the reader orders its other lanes after the
// acquiring lane the same way.
__device__ __forceinline__ void store_release(int *p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int load_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

template <typename T>
__device__ bool chase_wait_lane0(const ChaseArgs<T> &a, int s, int need) {
  // lane 0: wait until sweep s - 1 has completed `need` tasks (or finished); bounded
  if (s == 0) return true;
  const int *p = a.progress + (s - 1);
  volatile int *err = a.err;
  unsigned it = 0;
  while (load_acquire(p) < need) {
    if (*err != 0) return false;
    if (++it > kChaseSpinLimit) {
      atomicExch(a.err, 1);
      return false;
    }
  }
  return true;
}

// Householder reflector of x (lane l holds x_l, zero beyond len): returns v_l, tau and beta in all lanes.
template <typename T>
__device__ __forceinline__ T warp_reflector(T x, int len, T &tau, T &beta) {
  const int l = threadIdx.x & 31;
  const T ss = warp_sum((l >= 1) ? x * x : T(0));
  const T alpha = __shfl_sync(0xffffffffu, x, 0);
  T scale;
  if (ss == T(0) || len < 2) {
    tau = T(0);
    beta = alpha;
    scale = T(0);
  } else {
    beta = -copysign(sqrt(alpha * alpha + ss), alpha);
    tau = (beta - alpha) / beta;
    scale = T(1) / (alpha - beta);
  }
  return (l == 0) ? T(1) : ((l < len) ? x * scale : T(0));
}

// x[0..32) in every lane -> lane l returns sum over the lanes of x[l] (a 32 x 32 reduce-scatter by
// halving exchanges: 31 shuffles per lane; x is destroyed).
template <typename T>
__device__ __forceinline__ T warp_transpose_sum(T (&x)[kBand]) {
  const int l = threadIdx.x & 31;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    const bool up = (l & o) != 0;
#pragma unroll
    for (int i = 0; i < o; ++i) {
      const T send = up ? x[i] : x[i + o];
      const T keep = up ? x[i + o] : x[i];
      x[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
  return x[0];
}

// One warp per sweep: lane l holds row l of the 32 x 32 blocks B and D in registers (D row l read
// from its lower-triangle storage: A(c+l, c+j) for j <= l, A(c+j, c+l) above), so a task issues all
// its loads at once and synchronises the warp only to broadcast v and w through shared memory.
// Sweeps are dealt round-robin over all warps of a cooperative launch (sweep s to warp s mod W, each
// warp in increasing order).
constexpr int kChaseWarps = 4;

template <typename T>
struct ChaseSmem {
  T v[kBand], w[kBand], vprev[kBand];
};

template <typename T>
__device__ __forceinline__ void load_d_row(const ChaseArgs<T> &a, int c, int len, T (&drow)[kBand]) {
  const int l = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < kBand; ++j) {
    T x = T(0);
    if (l < len && j < len)
      x = (j <= l) ? __ldcg(a.A + (size_t)(c + l) + (size_t)(c + j) * a.lda)
                   : __ldcg(a.A + (size_t)(c + j) + (size_t)(c + l) * a.lda);
    drow[j] = x;
  }
}

// D <- H D H (H = I - tau v v^T) for the warp's D rows; the lower triangle goes back to A.
template <typename T>
__device__ __forceinline__ void chase_d_update(const ChaseArgs<T> &a, ChaseSmem<T> &S, int c, int len, T v, T tv,
                                               const T (&drow)[kBand]) {
  const int l = threadIdx.x & 31;
  T p = T(0);
#pragma unroll
  for (int j = 0; j < kBand; j += 4) {
    T vv[4];
    ld4(&S.v[j], vv);
#pragma unroll
    for (int q = 0; q < 4; ++q) p = fma(drow[j + q], vv[q], p);
  }
  p *= tv;
  const T om = T(-0.5) * tv * warp_sum(p * v);
  const T w = p + om * v;
  S.w[l] = w;
  __syncwarp();
#pragma unroll
  for (int j = 0; j < kBand; j += 4) {
    T vv[4], ww[4];
    ld4(&S.v[j], vv);
    ld4(&S.w[j], ww);
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (l < len && j + q <= l)
        a.A[(size_t)(c + l) + (size_t)(c + j + q) * a.lda] = drow[j + q] - v * ww[q] - w * vv[q];
  }
  __syncwarp();
}

template <typename T>
__global__ void __launch_bounds__(32 * kChaseWarps) sb2st_kernel(ChaseArgs<T> a) {
  constexpr int B = kBand;
  __shared__ __align__(16) ChaseSmem<T> smem[kChaseWarps];
  const int l = threadIdx.x & 31, wid = threadIdx.x >> 5;
  ChaseSmem<T> &S = smem[wid];
  const int n = a.n;
  const int nwarps = gridDim.x * kChaseWarps;
  const size_t blk_elems = (size_t)kL2 * kQ2Group;
  bool good = true;
  for (int s = blockIdx.x * kChaseWarps + wid; s < n - 1 && good; s += nwarps) {
    const int gS = s / kQ2Group, js = s - gS * kQ2Group;
    // ------------------------------------------------------------ task 0
    int ok = 0;
    if (l == 0) ok = chase_wait_lane0(a, s, 2) ? 1 : 0;
    ok = __shfl_sync(0xffffffffu, ok, 0);
    __syncwarp();
    if (!ok) { good = false; break; }
    const int c0 = s + 1;
    int len = min(B, n - c0);
    const T x0 = (l < len) ? __ldcg(a.A + (size_t)(c0 + l) + (size_t)s * a.lda) : T(0);
    T drow[B];
    load_d_row(a, c0, len, drow);
    if (l == 0) a.d[s] = __ldcg(a.A + (size_t)s + (size_t)s * a.lda);
    T tv, beta;
    T v = warp_reflector(x0, len, tv, beta);
    if (l == 0) a.e[s] = beta;
    S.v[l] = v;
    __syncwarp();
    if (tv != T(0)) chase_d_update(a, S, c0, len, v, tv, drow);
    {
      T *vb = a.V2 + ((size_t)gS * a.kmax + 0) * blk_elems + (size_t)js * kQ2Group + js;
      if (l < len) vb[(size_t)l * kQ2Group] = v;
      if (l == 0) a.tau2[((size_t)gS * a.kmax + 0) * kQ2Group + js] = tv;
    }
    S.vprev[l] = v;
    int len_prev = len;
    T tprev = tv;
    __syncwarp();   // every lane's stores of the task precede the releasing store
    if (l == 0) store_release(a.progress + s, 1);
    // ------------------------------------------------------------ tasks k >= 1
    int k = 1;
    for (int ck = s + 1 + B; ck < n; ck += B, ++k) {
      const int cp = ck - B;   // c_{k-1}
      len = min(B, n - ck);
      if (l == 0) ok = chase_wait_lane0(a, s, k + 2) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      __syncwarp();
      if (!ok) { good = false; break; }
      T brow[B];
#pragma unroll
      for (int j = 0; j < B; ++j)
        brow[j] = (l < len && j < len_prev) ? __ldcg(a.A + (size_t)(ck + l) + (size_t)(cp + j) * a.lda) : T(0);
      load_d_row(a, ck, len, drow);
      // B <- B H_{k-1} (lane-local row)
      if (tprev != T(0)) {
        T y = T(0);
#pragma unroll
        for (int j = 0; j < B; j += 4) {
          T vv[4];
          ld4(&S.vprev[j], vv);
#pragma unroll
          for (int q = 0; q < 4; ++q) y = fma(brow[j + q], vv[q], y);
        }
        y *= tprev;
#pragma unroll
        for (int j = 0; j < B; j += 4) {
          T vv[4];
          ld4(&S.vprev[j], vv);
#pragma unroll
          for (int q = 0; q < 4; ++q) brow[j + q] = fma(-y, vv[q], brow[j + q]);
        }
      }
      // H_k from the first column; the other columns of B <- H_k B
      v = warp_reflector(brow[0], len, tv, beta);
      brow[0] = (l == 0) ? beta : T(0);
      if (tv != T(0)) {
        T x[B];
#pragma unroll
        for (int j = 0; j < B; ++j) x[j] = v * brow[j];
        S.w[l] = tv * warp_transpose_sum(x);   // tau v^T B(:, l)
        __syncwarp();
#pragma unroll
        for (int j = 4; j < B; j += 4) {
          T ww[4];
          ld4(&S.w[j], ww);
#pragma unroll
          for (int q = 0; q < 4; ++q) brow[j + q] = fma(-v, ww[q], brow[j + q]);
        }
        {
          T ww[4];
          ld4(&S.w[0], ww);
#pragma unroll
          for (int q = 1; q < 4; ++q) brow[q] = fma(-v, ww[q], brow[q]);
        }
        __syncwarp();
      }
      if (l < len) {
#pragma unroll
        for (int j = 0; j < B; ++j)
          if (j < len_prev) a.A[(size_t)(ck + l) + (size_t)(cp + j) * a.lda] = brow[j];
      }
      S.v[l] = v;
      __syncwarp();
      if (tv != T(0)) chase_d_update(a, S, ck, len, v, tv, drow);
      {
        T *vb = a.V2 + ((size_t)gS * a.kmax + k) * blk_elems + (size_t)js * kQ2Group + js;
        if (l < len) vb[(size_t)l * kQ2Group] = v;
        if (l == 0) a.tau2[((size_t)gS * a.kmax + k) * kQ2Group + js] = tv;
      }
      S.vprev[l] = v;
      len_prev = len;
      tprev = tv;
      __syncwarp();
      if (l == 0) store_release(a.progress + s, k + 1);
    }
    if (!good) break;
    __syncwarp();
    if (l == 0) store_release(a.progress + s, kSweepDone);
  }
  if (l == 0 && a.status != nullptr && *(volatile int *)a.err != 0) atomicMax(a.status, (int)kDevIterCap);
}

template <typename T>
__global__ void last_diag_kernel(int n, const T *A, int lda, T *d) {
  d[n - 1] = A[(size_t)(n - 1) + (size_t)(n - 1) * lda];
}

// --------------------------------------------------------------------------------- stage-2 WY
// T factor of every stage-2 block: G = V^T V over the parallelogram, then the forward columnwise
// recurrence T(0:i, i) = -tau_i T(0:i, 0:i) G(0:i, i), T(i, i) = tau_i (LAPACK dlarft 'F', 'C').
template <typename T>
__global__ void __launch_bounds__(256) q2_tfactor_kernel(int n, int kmax, const T *V2, const T *tau2, T *T2) {
  constexpr int g = kQ2Group;
  __shared__ T Vs[kL2][g + 1];
  __shared__ T Gs[g][g + 1];
  __shared__ T Ts[g][g + 1];
  __shared__ T ts[g];
  const int blk = blockIdx.x, gS = blk / kmax, k = blk - gS * kmax;
  const int s0 = gS * g;
  if (s0 > n - 2 || k > (n - 2 - s0) / kBand) return;
  const int t = threadIdx.x;
  const T *V = V2 + (size_t)blk * kL2 * g;   // row-major kL2 x g
  for (int idx = t; idx < kL2 * g; idx += 256) Vs[idx / g][idx % g] = V[idx];
  if (t < g) ts[t] = tau2[(size_t)blk * g + t];
  for (int idx = t; idx < g * g; idx += 256) Ts[idx % g][idx / g] = T(0);
  __syncthreads();
  for (int idx = t; idx < g * g; idx += 256) {
    const int i = idx % g, j = idx / g;
    T acc = T(0);
    for (int r = 0; r < kL2; ++r) acc = fma(Vs[r][i], Vs[r][j], acc);
    Gs[i][j] = acc;
  }
  __syncthreads();
  for (int i = 0; i < g; ++i) {
    T v = T(0);
    if (t < i) {
      for (int q = t; q < i; ++q) v = fma(Ts[t][q], Gs[q][i], v);
      v *= -ts[i];
    }
    __syncthreads();
    if (t < i) Ts[t][i] = v;
    if (t == 0) Ts[i][i] = ts[i];
    __syncthreads();
  }
  T *To = T2 + (size_t)blk * g * g;   // row-major g x g (zeros below the diagonal)
  for (int idx = t; idx < g * g; idx += 256) To[idx] = Ts[idx / g][idx % g];
}

// Z <- Q2 Z. Q2 is the product, in sweep order, of the blocks P(S, k) = I - V T V^T of the sweep
// groups S; within a group the blocks are applied from chain position 0 upwards (reflectors of one
// sweep act on disjoint rows and commute, and H(s, k) must precede H(s', k - 1) for s < s'), the
// groups from last to first. Block (S, k) covers rows [32 (S + k) + 1, 32 (S + k) + 63]; it overlaps
// blocks k - 2 .. k of group S + 1, so it may run once group S + 1 has finished block k on the same
// columns. Work items (group, strip of kQ2Cols columns) are dealt to the co-resident CTAs of a
// cooperative launch, last group first; every thread owns one column and keeps its 63-row window in
// registers, the block's V and T are staged in shared memory. Waits are bounded.
constexpr int kQ2Cols = 256;   // columns per work item (two per thread)

template <typename T>
struct Q2Args {
  int n, ncols, kmax, ngrp, nstrip;
  const T *V2, *T2;
  T *Z;
  int ldz;
  int *progress;   // [ngrp * nstrip]: blocks finished per item
  int *counter;    // next item to take
  int *err;
  int *status;
};

// Two columns per thread (t and t + kQ2Cols/2): every 16-byte read of a V row feeds 8 FMAs. The
// 63-row window of the item's columns slides down the group's blocks in shared memory: block k
// keeps rows 32..62 of block k - 1 (shifted to 0..30) and loads rows 31..62; after the block, rows
// 0..31 are final for this group and go back to global memory. Global accesses are coalesced (a
// warp covers 32 consecutive rows of one column); the window rows are padded to avoid bank
// conflicts of the transposed accesses.
constexpr int kQ2Pad = kQ2Cols + 1;

template <typename T>
__global__ void __launch_bounds__(kQ2Cols / 2) q2_apply_kernel(Q2Args<T> a) {
  constexpr int g = kQ2Group, L = kL2, NT = kQ2Cols / 2, NW = NT / 32;
  extern __shared__ __align__(16) unsigned char q2_smem[];
  T (*Vs)[g] = reinterpret_cast<T (*)[g]>(q2_smem);                                  // [L][g]
  T (*Ts)[g] = reinterpret_cast<T (*)[g]>(q2_smem + sizeof(T) * L * g);              // [g][g]
  T (*Zs)[kQ2Pad] = reinterpret_cast<T (*)[kQ2Pad]>(q2_smem + sizeof(T) * (L + g) * g);   // [L][cols + 1]
  __shared__ int ok;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int nitems = a.ngrp * a.nstrip;
  __shared__ int s_item;
  while (true) {
    // items are taken in index order from a counter: an item waits only on the item nstrip before
    // it, which a running CTA took earlier
    if (t == 0) s_item = atomicAdd(a.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= nitems) break;
    const int gS = a.ngrp - 1 - item / a.nstrip;
    const int p = item - (item / a.nstrip) * a.nstrip;
    const int cbase = p * kQ2Cols;
    const int ncol = min(kQ2Cols, a.ncols - cbase);
    const int s0 = gS * g;
    int *prog_me = a.progress + (size_t)gS * a.nstrip + p;
    const int *prog_prev = (gS + 1 < a.ngrp) ? a.progress + (size_t)(gS + 1) * a.nstrip + p : nullptr;
    const int kmx = (s0 <= a.n - 2) ? (a.n - 2 - s0) / kBand : -1;
    T *Zb = a.Z + (size_t)cbase * a.ldz;
    bool good = true;
    for (int k = 0; k <= kmx; ++k) {
      if (t == 0) {
        int r = 1;
        if (prog_prev != nullptr) {
          volatile int *err = a.err;
          unsigned it = 0;
          while (load_acquire(prog_prev) < k + 1) {
            if (*err != 0) { r = 0; break; }
            if (++it > kChaseSpinLimit) { atomicExch(a.err, 1); r = 0; break; }
          }
        }
        ok = r;
      }
      __syncthreads();
      if (!ok) { good = false; break; }
      const size_t blk = (size_t)gS * a.kmax + k;
      const T *V = a.V2 + blk * L * g;    // row-major L x g
      const T *Tf = a.T2 + blk * g * g;   // row-major g x g
      T *vflat = &Vs[0][0];
      T *tflat = &Ts[0][0];
      for (int idx = t; idx < L * g; idx += NT) vflat[idx] = __ldcg(V + idx);
      for (int idx = t; idx < g * g; idx += NT) tflat[idx] = __ldcg(Tf + idx);
      const int r0 = s0 + 1 + k * kBand;
      const int rows = min(L, a.n - r0);
      // new window rows: all of them for the first block, rows 31..62 afterwards
      const int jlo = (k == 0) ? 0 : L - kBand;
      for (int c = warp; c < kQ2Cols; c += NW) {
        const T *zc = Zb + (size_t)c * a.ldz + r0;
        for (int j = jlo + lane; j < L; j += 32) Zs[j][c] = (c < ncol && j < rows) ? __ldcg(zc + j) : T(0);
      }
      __syncthreads();
      T w0[g], w1[g];
#pragma unroll
      for (int i = 0; i < g; ++i) {
        w0[i] = T(0);
        w1[i] = T(0);
      }
#pragma unroll 1
      for (int r = 0; r < L; ++r) {
        const T z0 = Zs[r][t], z1 = Zs[r][t + NT];
#pragma unroll
        for (int i = 0; i < g; i += 4) {
          T v[4];
          ld4(&Vs[r][i], v);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            w0[i + q] = fma(v[q], z0, w0[i + q]);
            w1[i + q] = fma(v[q], z1, w1[i + q]);
          }
        }
      }
      // w <- T w (T upper, zeros below): in place in ascending order of the output row
#pragma unroll
      for (int i = 0; i < g; ++i) {
        T a0 = T(0), a1 = T(0);
#pragma unroll
        for (int q = (i / 4) * 4; q < g; q += 4) {
          T tv[4];
          ld4(&Ts[i][q], tv);
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            a0 = fma(tv[u], w0[q + u], a0);
            a1 = fma(tv[u], w1[q + u], a1);
          }
        }
        w0[i] = a0;
        w1[i] = a1;
      }
#pragma unroll 1
      for (int r = 0; r < L; ++r) {
        T a0 = Zs[r][t], a1 = Zs[r][t + NT];
#pragma unroll
        for (int i = 0; i < g; i += 4) {
          T v[4];
          ld4(&Vs[r][i], v);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            a0 = fma(-v[q], w0[i + q], a0);
            a1 = fma(-v[q], w1[i + q], a1);
          }
        }
        Zs[r][t] = a0;
        Zs[r][t + NT] = a1;
      }
      __syncthreads();
      // rows 0..31 are final for this group (all rows after its last block)
      const int jhi = (k == kmx) ? rows : min(rows, kBand);
      for (int c = warp; c < ncol; c += NW) {
        T *zc = Zb + (size_t)c * a.ldz + r0;
        for (int j = lane; j < jhi; j += 32) zc[j] = Zs[j][c];
      }
      __syncthreads();
      if (t == 0) store_release(prog_me, k + 1);
      if (k < kmx) {
        // slide: rows 32..62 -> 0..30
        for (int idx = t; idx < (L - kBand) * kQ2Cols; idx += NT) {
          const int j = idx / kQ2Cols, c = idx - j * kQ2Cols;
          Zs[j][c] = Zs[j + kBand][c];
        }
      }
    }
    if (!good) break;
    if (t == 0) store_release(prog_me, kSweepDone);
    __syncthreads();
  }
  if (t == 0 && a.status != nullptr && *(volatile int *)a.err != 0) atomicMax(a.status, (int)kDevIterCap);
}

template <typename T>
constexpr size_t q2_smem_bytes() {
  return sizeof(T) * ((size_t)(kL2 + kQ2Group) * kQ2Group + (size_t)kL2 * kQ2Pad);
}

template <typename T>
int coop_ctas(const void *fn, int threads, size_t smem) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
  return sms * std::max(per_sm, 0);
}

}  // namespace

// ----------------------------------------------------------------------------------- host side
template <typename T>
TwoStageLayout twostage_layout(int n) {
  TwoStageLayout L;
  const int b = kBand;
  L.n = n;
  L.kmax = std::max(1, (n - 2) / b + 1);
  L.ngrp = std::max(1, ceil_div(std::max(n - 1, 1), kQ2Group));
  L.gmax = 4096;
  const int npan = ceil_div(n, b) + 1;
  size_t o = 0;
  auto take = [&](size_t cnt) {
    size_t r = o;
    o += (cnt + 31) / 32 * 32;   // 128-byte alignment for FP32, 256 for FP64
    return r;
  };
  L.tau1 = take((size_t)n);
  L.T1 = take((size_t)npan * b * b);
  L.X1 = take((size_t)n * b);   // X1, X, X2 contiguous (n * b is a multiple of 32): [V | W | V]
  L.X = take((size_t)n * b);
  L.X2 = take((size_t)n * b);
  L.G = take((size_t)b * b);
  L.G2 = take((size_t)b * b);
  L.M = take((size_t)b * b);
  L.split_elems = std::max((size_t)64 * b * b, (size_t)8 * n * b);   // split-K partials
  L.split = take(L.split_elems);
  L.part = take((size_t)2 * L.gmax * b);
  L.top = take((size_t)2 * b);
  L.V2 = take((size_t)L.ngrp * L.kmax * kL2 * kQ2Group);
  L.tau2 = take((size_t)L.ngrp * L.kmax * kQ2Group);
  L.T2 = take((size_t)L.ngrp * L.kmax * kQ2Group * kQ2Group);
  // integers: GridBar (4 ints), chase error word, progress[n]
  // GridBar, error word, work counter; chase progress[n]; Q2 anti-diagonal starts and progress
  const size_t nint = 16 + (size_t)n + 2 * (size_t)L.ngrp + 2 + (size_t)L.ngrp * (size_t)(ceil_div(n, 128) + 1);
  L.ints = take((nint * sizeof(int) + sizeof(T) - 1) / sizeof(T));
  L.total = o;
  return L;
}

template <typename T>
size_t twostage_work_size(int n) {
  return twostage_layout<T>(n).total;
}

template <typename T>
static void sy2sb_lower(cudaStream_t s, int n, T *A, int lda, T *V1, int ldv, T *w, const TwoStageLayout &L,
                        int *status) {
  const int b = kBand;
  T *tau1 = w + L.tau1, *T1 = w + L.T1, *X1 = w + L.X1, *X = w + L.X, *X2 = w + L.X2, *Gm = w + L.G, *G2 = w + L.G2,
    *M = w + L.M, *split = w + L.split, *part = w + L.part, *top = w + L.top;
  GridBar *bar = reinterpret_cast<GridBar *>(w + L.ints);
  ensure_dyn_smem((const void *)panel_qr_kernel<T>, 200 * 1024);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  for (int p0 = 0, ip = 0;; p0 += b, ++ip) {
    const int m = n - p0 - b;
    if (m < 2) break;
    const int kr = std::min(m, b);
    T *P = A + (p0 + b) + (size_t)p0 * lda;
    T *Vp = V1 + (p0 + b) + (size_t)p0 * ldv;
    // rows per CTA >= 64 (so the top kr rows live in CTA 0); shared panel <= 200 KB
    int G = std::max(1, std::min(m / 64, sms));
    while (G < sms && (size_t)ceil_div(m, G) * b * sizeof(T) > 160 * 1024) ++G;
    const int R = ceil_div(m, G);
    const size_t smem = (size_t)R * b * sizeof(T);
    cudaMemsetAsync(bar, 0, sizeof(GridBar), s);
    PanelQrArgs<T> qa{P, lda, Vp, ldv, tau1 + p0, m, b, kr, R, part, top, bar, status};
    void *args[] = {&qa};
    KernelTimer kt(s);
    cudaLaunchCooperativeKernel((const void *)panel_qr_kernel<T>, dim3(G), dim3(kQrThreads), args, smem, s);
    count_launch();
    kt.done(kPhKPanelQr, 2.0 * m * b * sizeof(T));   // panel read and written once
    T *Tp = T1 + (size_t)ip * b * b;
    gemm<T>(s, 'T', 'N', kr, kr, m, T(1), Vp, ldv, Vp, ldv, T(0), Gm, kr, 0, split, L.split_elems);
    larft<T>(s, kr, Gm, tau1 + p0, Tp);
    T *A22 = A + (p0 + b) + (size_t)(p0 + b) * lda;
    // X = A22 V T; W = X - 1/2 V (T^T V^T X); A22 -= W V^T + V W^T (lower), then mirrored
    gemm<T>(s, 'N', 'N', m, kr, m, T(1), A22, lda, Vp, ldv, T(0), X1, n, 0, split, L.split_elems);
    gemm<T>(s, 'N', 'N', m, kr, kr, T(1), X1, n, Tp, kr, T(0), X, n, kBUpper);
    gemm<T>(s, 'T', 'N', kr, kr, m, T(1), Vp, ldv, X, n, T(0), G2, kr, 0, split, L.split_elems);
    gemm<T>(s, 'T', 'N', kr, kr, kr, T(1), Tp, kr, G2, kr, T(0), M, kr, kALower);
    gemm<T>(s, 'N', 'N', m, kr, kr, T(-0.5), Vp, ldv, M, kr, T(1), X, n);
    if (kr == b) {
      // one rank-2b update: [V | W] [W | V]^T with V copied beside W on both sides
      cudaMemcpy2DAsync(X1, sizeof(T) * n, Vp, sizeof(T) * ldv, sizeof(T) * m, kr, cudaMemcpyDeviceToDevice, s);
      cudaMemcpy2DAsync(X2, sizeof(T) * n, Vp, sizeof(T) * ldv, sizeof(T) * m, kr, cudaMemcpyDeviceToDevice, s);
      gemm<T>(s, 'N', 'T', m, m, 2 * kr, T(-1), X1, n, X, n, T(1), A22, lda, kCLower);
    } else {
      gemm<T>(s, 'N', 'T', m, m, kr, T(-1), X, n, Vp, ldv, T(1), A22, lda, kCLower);
      gemm<T>(s, 'N', 'T', m, m, kr, T(-1), Vp, ldv, X, n, T(1), A22, lda, kCLower);
    }
    if (m > b) copy_lower_to_upper<T>(s, m, A22, lda);
  }
}

template <typename T>
void twostage_reduce(cudaStream_t s, int n, T *A, int lda, T *d, T *e, T *V1, int ldv, T *work, int *status) {
  if (n <= 0) return;
  if (n == 1) {
    last_diag_kernel<T><<<1, 1, 0, s>>>(n, A, lda, d);
    count_launch();
    return;
  }
  const TwoStageLayout L = twostage_layout<T>(n);
  copy_lower_to_upper<T>(s, n, A, lda);   // the panel products read A22 as a full symmetric matrix
  sy2sb_lower<T>(s, n, A, lda, V1, ldv, work, L, status);
  // stage 2
  T *V2 = work + L.V2, *tau2 = work + L.tau2;
  int *ints = reinterpret_cast<int *>(work + L.ints);
  int *err = ints + 8;
  int *progress = ints + 16;
  cudaMemsetAsync(V2, 0, sizeof(T) * (size_t)L.ngrp * L.kmax * kL2 * kQ2Group, s);
  cudaMemsetAsync(tau2, 0, sizeof(T) * (size_t)L.ngrp * L.kmax * kQ2Group, s);
  cudaMemsetAsync(ints + 8, 0, sizeof(int) * (8 + (size_t)n), s);
  static int g_chase = 0;
  if (g_chase == 0) g_chase = coop_ctas<T>((const void *)sb2st_kernel<T>, 32 * kChaseWarps, 0);
  // useful concurrency: sweeps run two tasks apart, about n / (2 b) of them at once (one per warp)
  const int want_warps = std::min(n - 1, (n - 1) / (2 * kBand) + 8);
  const int G = std::max(1, std::min(g_chase, ceil_div(want_warps, kChaseWarps)));
  ChaseArgs<T> ca{A, lda, n, L.kmax, d, e, V2, tau2, progress, err, status};
  void *args[] = {&ca};
  KernelTimer kt(s);
  cudaLaunchCooperativeKernel((const void *)sb2st_kernel<T>, dim3(G), dim3(32 * kChaseWarps), args, 0, s);
  {
    double tasks = 0.0;   // Householder tasks of all sweeps
    for (int sw = 0; sw < n - 1; ++sw) tasks += 1.0 + std::max(0, (n - 2 - sw) / kBand);
    kt.done(kPhKChase, tasks);
  }
  last_diag_kernel<T><<<1, 1, 0, s>>>(n, A, lda, d);
  q2_tfactor_kernel<T><<<L.ngrp * L.kmax, 256, 0, s>>>(n, L.kmax, V2, tau2, work + L.T2);
  count_launch(3);
}

template <typename T>
void twostage_back(cudaStream_t s, int n, int k, T *Z, int ldz, const T *V1, int ldv, T *work, int *status) {
  if (n <= 1 || k <= 0) return;
  const TwoStageLayout L = twostage_layout<T>(n);
  const int b = kBand;
  {
    const int nstrip = ceil_div(k, kQ2Cols);
    int *ints = reinterpret_cast<int *>(work + L.ints);
    int *err = ints + 8;
    int *counter = ints + 9;
    int *prog = ints + 16 + n;   // after the chase's progress words
    cudaMemsetAsync(err, 0, 2 * sizeof(int), s);
    cudaMemsetAsync(prog, 0, sizeof(int) * (size_t)L.ngrp * nstrip, s);
    ensure_dyn_smem((const void *)q2_apply_kernel<T>, (int)q2_smem_bytes<T>());
    static int g_q2 = 0;   // co-resident CTAs (the same on every GB300)
    if (g_q2 == 0) g_q2 = coop_ctas<T>((const void *)q2_apply_kernel<T>, kQ2Cols / 2, q2_smem_bytes<T>());
    const int G = std::max(1, std::min(g_q2, L.ngrp * nstrip));
    Q2Args<T> qa{n, k, L.kmax, L.ngrp, nstrip, work + L.V2, work + L.T2, Z, ldz, prog, counter, err, status};
    void *args[] = {&qa};
    KernelTimer kt(s);
    cudaLaunchCooperativeKernel((const void *)q2_apply_kernel<T>, dim3(G), dim3(kQ2Cols / 2), args, q2_smem_bytes<T>(), s);
    count_launch();
    kt.done(kPhKBackQ2, 2.0 * (double)n * n * k);   // algorithmic FLOPs of applying Q2 to k vectors
  }
  // Z <- P_p Z for the stage-1 panels from last to first
  int last = -1;
  for (int p0 = 0;; p0 += b) {
    if (n - p0 - b < 2) break;
    last = p0;
  }
  T *M = work + L.X1, *M2 = work + L.X;   // kr x k each fits in n x b (k <= n)
  T *split = work + L.split;
  for (int p0 = last, ip = last / b; p0 >= 0; p0 -= b, --ip) {
    const int m = n - p0 - b;
    const int kr = std::min(m, b);
    const T *Vp = V1 + (p0 + b) + (size_t)p0 * ldv;
    const T *Tp = work + L.T1 + (size_t)ip * b * b;
    T *Zp = Z + (p0 + b);
    gemm<T>(s, 'T', 'N', kr, k, m, T(1), Vp, ldv, Zp, ldz, T(0), M, kr, 0, split, L.split_elems);
    gemm<T>(s, 'N', 'N', kr, k, kr, T(1), Tp, kr, M, kr, T(0), M2, kr, kAUpper);
    gemm<T>(s, 'N', 'N', m, k, kr, T(-1), Vp, ldv, M2, kr, T(1), Zp, ldz);
  }
}

template TwoStageLayout twostage_layout<float>(int);
template TwoStageLayout twostage_layout<double>(int);
template size_t twostage_work_size<float>(int);
template size_t twostage_work_size<double>(int);
template void twostage_reduce<float>(cudaStream_t, int, float *, int, float *, float *, float *, int, float *, int *);
template void twostage_reduce<double>(cudaStream_t, int, double *, int, double *, double *, double *, int, double *,
                                      int *);
template void twostage_back<float>(cudaStream_t, int, int, float *, int, const float *, int, float *, int *);
template void twostage_back<double>(cudaStream_t, int, int, double *, int, const double *, int, double *, int *);

}  // namespace dg
