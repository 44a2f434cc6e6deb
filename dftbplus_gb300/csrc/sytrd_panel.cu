// Panels of the one-stage tridiagonalisation (sytrd_lower in linalg.cu) with the trailing matrix
// held on chip: one cooperative launch per panel of 32 columns, one CTA of 512 threads per SM.
//
// The symmetric matrix-vector product y = A22 v of every column of a panel reads the same data: the
// trailing matrix as it was when the panel started (the panel's own reflectors enter through the
// V W^T + W V^T corrections, LAPACK dlatrd). So the tiles are cut on a grid fixed for the whole
// panel (64 x 64 tiles of A(p0:n, p0:n), lower triangle) instead of one that moves with the column;
// rows and columns a column no longer touches are masked by zeros in v. Each CTA keeps the first of
// its tiles resident in shared memory for the whole panel (loaded once by TMA) and streams the rest
// through a three-stage TMA ring that runs on across column boundaries (the data does not change,
// so the next column's first tiles arrive while the grid barriers and row phases run).
//
// Per column j two grid barriers separate two phases:
//   R(j): finish W(:, j-1) = tau (y - V dW - W dV) + alpha v with alpha = -tau/2 w^T v computed as
//         -tau^2/2 (v^T A22 v - 2 dV.dW) from per-CTA partials of v^T A22 v (no barrier of its own);
//         update column j (A(j:n, j) -= V W(j,:)^T + W V(j,:)^T, with W(j, j-1) recomputed by every
//         CTA); per-CTA partials of ||A(j+2:n, j)||^2 and of V^T a, W^T a.
//   B(j): reflector (dlarfg) from the partials in every CTA; v staged in shared memory; the dots
//         W^T v, V^T v from their partials; tile products into the partial slots P[R][C] and the
//         CTA's partial of v^T A22 v.
// Every cross-CTA sum adds per-CTA partials in a fixed order, so results are deterministic.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdint>
#include <cstring>

#include "gridsync.cuh"
#include "linalg.cuh"
#include "tcgen05.cuh"
#include "tma.cuh"

namespace dg {

namespace {

constexpr int kTile = 64;           // tile edge
constexpr int kPb = 32;             // panel width (same as the one-stage panels in linalg.cu)
constexpr int kThreads = 512;
// v elements staged per thread: trailing size up to 12,288 (FP32) or 6,144 (FP64)
template <typename T>
constexpr int kVPer = sizeof(T) == 8 ? 12 : 24;
constexpr int kGroups = 4;          // tile groups per CTA
constexpr int kGThreads = kThreads / kGroups;
constexpr int kMaxSlots = 16;       // tile slots (at least one per group)
constexpr int kMaxK = 256;          // tiles per CTA
// per group two buffers of row partials (4 warps x 64) and diagonal-tile column totals (64)
constexpr int kRed = kGroups * 2 * (kGroups * kTile + kTile);

template <typename T>
struct Args {
  T *A;
  int lda, n, p0, nbp, nslot;
  T *Vp, *Wp, *P, *dots, *part, *vpart, *dpart;
  T *V, *d, *e, *tau;
  int ldv;
  GridBar *bar;
  unsigned base;   // the barrier counter when the launch starts
  int *status;
};

__device__ __forceinline__ void mbar_arrive_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tma_load_tile(uint32_t dst, const void *map, int x, int y, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(map), "r"(x), "r"(y), "r"(mbar)
      : "memory");
}

template <typename T>
__device__ __forceinline__ void cp_async_elem(uint32_t dst, const T *src, bool valid) {
  if constexpr (sizeof(T) == 4)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(valid ? 4 : 0) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(dst), "l"(src), "r"(valid ? 8 : 0) : "memory");
}

__device__ __forceinline__ void cp_async_arrive(uint32_t mbar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(mbar) : "memory");
}

// Bounded wait; on a timeout the error word is set (the grid barriers then stop waiting) and the
// thread waits once more, again bounded, for the copy in flight before it goes on.
__device__ __forceinline__ void slot_wait(uint32_t mbar, uint32_t parity, GridBar *bar) {
  if (!mbar_wait(mbar, parity)) {
    atomicExch(&bar->err, 1);
    mbar_wait(mbar, parity);
  }
}

// Sum over the 8 lanes of a row group (lanes differing in bits 0..2), fixed tree.
template <typename T>
__device__ __forceinline__ T sum8(T v) {
  v += __shfl_xor_sync(0xffffffffu, v, 4);
  v += __shfl_xor_sync(0xffffffffu, v, 2);
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  return v;
}

// Eight per-lane values summed over the 32 lanes of a warp: lane l returns the total of value
// (l >> 2) & 7 (9 shuffles instead of 40).
template <typename T>
__device__ __forceinline__ T transpose_sum8(const T (&v)[8]) {
  const int l = threadIdx.x & 31;
  const bool b4 = l & 16, b3 = l & 8, b2 = l & 4;
  T w[4], x[2];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const T send = b4 ? v[k] : v[k + 4];
    const T keep = b4 ? v[k + 4] : v[k];
    w[k] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const T send = b3 ? w[k] : w[k + 2];
    const T keep = b3 ? w[k + 2] : w[k];
    x[k] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
  T y = (b2 ? x[1] : x[0]) + __shfl_xor_sync(0xffffffffu, b2 ? x[0] : x[1], 4);
  y += __shfl_xor_sync(0xffffffffu, y, 2);
  y += __shfl_xor_sync(0xffffffffu, y, 1);
  return y;
}

// Lower-triangle tile index -> (row tile, column tile).
__device__ __forceinline__ void tile_of(int idx, int &r, int &c) {
  r = (int)((sqrtf(8.f * (float)idx + 1.f) - 1.f) * 0.5f);
  while ((r + 1) * (r + 2) / 2 <= idx) ++r;
  while (r * (r + 1) / 2 > idx) --r;
  c = idx - r * (r + 1) / 2;
}

// Eight per-lane values summed over the 16 lanes of a half warp (lanes differing in bits 0..3):
// lane l returns the total of value (l >> 1) & 7 (8 shuffles).
template <typename T>
__device__ __forceinline__ T transpose_sum8_16(const T (&v)[8]) {
  const int l = threadIdx.x & 31;
  const bool b3 = l & 8, b2 = l & 4, b1 = l & 2;
  T w[4], x[2];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const T send = b3 ? v[k] : v[k + 4];
    const T keep = b3 ? v[k + 4] : v[k];
    w[k] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const T send = b2 ? w[k] : w[k + 2];
    const T keep = b2 ? w[k + 2] : w[k];
    x[k] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
  }
  T y = (b1 ? x[1] : x[0]) + __shfl_xor_sync(0xffffffffu, b1 ? x[0] : x[1], 2);
  y += __shfl_xor_sync(0xffffffffu, y, 1);
  return y;
}

// Four consecutive elements from 16-byte aligned shared memory.
__device__ __forceinline__ void lds4(const float *p, float (&v)[4]) {
  const float4 q = *reinterpret_cast<const float4 *>(p);
  v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
}
__device__ __forceinline__ void lds4(const double *p, double (&v)[4]) {
  const double2 q0 = *reinterpret_cast<const double2 *>(p), q1 = *reinterpret_cast<const double2 *>(p + 2);
  v[0] = q0.x, v[1] = q0.y, v[2] = q1.x, v[3] = q1.y;
}

__device__ __forceinline__ void group_sync(int g) {
  asm volatile("bar.sync %0, %1;" ::"r"(1 + g), "r"(kGThreads) : "memory");
}

template <typename T, bool kTma>
__global__ void __launch_bounds__(kThreads, 1) sytrd_panel_resident_kernel(const __grid_constant__ CUtensorMap tmap,
                                                                           Args<T> a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ uint64_t s_mbar[kMaxSlots];
  __shared__ int s_tile[kMaxK];
  __shared__ T sh[64];
  __shared__ T cW[kPb], cV[kPb], sdW[kPb], sdV[kPb];
  // [2]: vs with v = vs x for the staged x (x(j+1) = alpha - beta); [4]: dlarfg's scale
  __shared__ T s_scal[5];

  const int n = a.n, G = gridDim.x, b = blockIdx.x, t = threadIdx.x;
  const int lane = t & 31, lane8 = t & 7, rloc = t >> 3;
  const int o = a.p0, mt = n - o;
  const int nt = (mt + kTile - 1) / kTile, ntiles = nt * (nt + 1) / 2;
  const int vlen = nt * kTile;
  T *slots = reinterpret_cast<T *>(smem_raw);
  T *vall = slots + (size_t)a.nslot * kTile * kTile;
  T *red = vall + vlen;
  const unsigned nb = (unsigned)G;
  unsigned epoch = 0;   // barriers of this launch
  constexpr uint32_t kTileBytes = kTile * kTile * sizeof(T);

  // This CTA's tiles b, b + G, ... (k = 0 .. K-1) are shared among four groups of 128 threads
  // (group g: k = g, g + 4, ...). Each group has its share of the slots: all its tiles resident when
  // they fit, otherwise a ring through which its tiles stream every column.
  const int K = (b < ntiles) ? (ntiles - 1 - b) / G + 1 : 0;
  for (int k = t; k < K; k += kThreads) {
    int tr, tc;
    tile_of(b + k * G, tr, tc);
    s_tile[k] = (tr << 16) | tc;
  }
  const int g = t >> 7, tg = t & (kGThreads - 1), wg = tg >> 5;
  const int ns = a.nslot / kGroups + (g < a.nslot % kGroups ? 1 : 0);
  const int sbase = g * (a.nslot / kGroups) + min(g, a.nslot % kGroups);
  const int Kg = (K > g) ? (K - 1 - g) / kGroups + 1 : 0;
  const bool gres = Kg <= ns;
  const long long glen = (long long)a.nbp * Kg;
  T *gslots = slots + (size_t)sbase * kTile * kTile;
  T *gred = red + g * 2 * (kGroups * kTile + kTile);   // [2][rows 4 x 64 | columns 64]
  auto gbar = [&](int s) { return smem_u32(&s_mbar[sbase + s]); };
  auto gissue = [&](int kk, int s) {
    const int packed = s_tile[g + kGroups * kk];
    const int r0 = o + kTile * (packed >> 16), c0 = o + kTile * (packed & 0xffff);
    T *slot = gslots + (size_t)s * kTile * kTile;
    if constexpr (kTma) {
      if (tg == 0) {
        mbar_arrive_tx(gbar(s), kTileBytes);
        tma_load_tile(smem_u32(slot), &tmap, r0, c0, gbar(s));
      }
    } else {
#pragma unroll 8
      for (int q = 0; q < kTile * kTile / kGThreads; ++q) {
        const int el = tg + kGThreads * q, i = el & (kTile - 1), c = el >> 6;
        const int r = r0 + i, cc = c0 + c;
        const bool ok = r < n && cc < n;
        cp_async_elem<T>(smem_u32(slot + el), ok ? a.A + r + (size_t)cc * a.lda : a.A, ok);
      }
      cp_async_arrive(gbar(s));
    }
  };
  if (t == 0) {
    for (int s = 0; s < a.nslot; ++s) mbar_init(smem_u32(&s_mbar[s]), kTma ? 1 : kGThreads);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (gres) {
    for (int kk = 0; kk < Kg; ++kk) gissue(kk, kk);
  } else {
    for (int u = 0; u < ns; ++u) gissue(u % Kg, u);
  }

  // rows of the row phases: a contiguous block per CTA, 8 lanes per row, 64 rows per pass
  const int RB = (mt + G - 1) / G;
  const int row0 = o + b * RB, row1 = min(n, row0 + RB);

  for (int jj = 0; jj <= a.nbp; ++jj) {
    const int j = o + jj;
    const bool last = jj == a.nbp;   // only W(:, nbp - 1) remains
    T *colj = a.A + (size_t)j * a.lda;
    // ------------------------------------------------------------------------------------- R
    {
      const int qn = jj - 1;
      // Prologue (jj > 0), by warp 0 once the first rows' loads are in flight: alpha of column
      // jp = j - 1 and W(j, qn), identical in every CTA. P and the v^T A22 v partials hold products
      // with the staged x = v / vs (vs of column jp). Leaves cW/cV (W(j,:), V(j,:)), sdW/sdV (the
      // dots of column jp) and s_scal[0..1] = {alpha, tau}.
      T sig = T(0), pdv[4] = {T(0), T(0), T(0), T(0)}, pdw[4] = {T(0), T(0), T(0), T(0)};
      T alpha = T(0), tp = T(0), vs = T(0);
      if (jj == 0 && t < kPb) {
        cW[t] = T(0);
        cV[t] = T(0);
      }
      for (int rb = row0; rb < row1; rb += kThreads / 8) {   // CTA-uniform trip count
        const int r = rb + rloc;
        const bool in = r < row1, act = in && !last && r >= j;
        T ys = T(0), vpn = T(0), cj = T(0), vq[4], wq[4];
        if (jj > 0 && in) {
          const int rr = r - o, Rr = rr / kTile, ir = rr % kTile;
#pragma unroll 8
          for (int C = lane8; C < nt; C += 8) ys += __ldcg(a.P + ((size_t)Rr * nt + C) * kTile + ir);
          vpn = __ldcg(a.Vp + r + (size_t)qn * n);
        }
        if (act) cj = __ldcg(colj + r);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int q = lane8 + 8 * i;
          vq[i] = (in && q < qn) ? __ldcg(a.Vp + r + (size_t)q * n) : T(0);
          wq[i] = (in && q < qn) ? __ldcg(a.Wp + r + (size_t)q * n) : T(0);
        }
        if (jj > 0 && rb == row0) {
          if (t < 32) {
            const int jp = j - 1;
            const T tpw = __ldcg(a.tau + jp), vsw = s_scal[2];
            T x = T(0), yq = T(0), ldW = T(0), ldV = T(0), lw = T(0), lv = T(0);
            for (int i = lane; i < G; i += 32) x += __ldcg(a.vpart + i);
            const int rr = j - o, Rj = rr / kTile, ij = rr % kTile;
            for (int C = lane; C < nt; C += 32) yq += __ldcg(a.P + ((size_t)Rj * nt + C) * kTile + ij);
            if (lane < qn) {
              ldW = __ldcg(a.dots + lane), ldV = __ldcg(a.dots + kPb + lane);
              lw = __ldcg(a.Wp + j + (size_t)lane * n);
              lv = __ldcg(a.Vp + j + (size_t)lane * n);
            }
            yq = vsw * yq - (lv * ldW + lw * ldV);
            const T vav = vsw * vsw * warp_sum(x), yj = warp_sum(yq), ddot = warp_sum(ldV * ldW);
            const T al = T(-0.5) * tpw * (tpw * (vav - T(2) * ddot));
            if (lane == qn) {
              lw = tpw * yj + al;   // v_{j-1}(j) = 1
              lv = T(1);
            }
            cW[lane] = lw;
            cV[lane] = lv;
            sdW[lane] = ldW;
            sdV[lane] = ldV;
            if (lane == 0) {
              s_scal[0] = al;
              s_scal[1] = tpw;
            }
          }
          __syncthreads();
        }
        if (jj > 0) {
          alpha = s_scal[0];
          tp = s_scal[1];
          vs = s_scal[2];
        }
        if (rb + 4 * (t >> 5) >= row1) continue;   // no row of this warp in this pass (warp-uniform)
        T wnew = T(0);
        if (jj > 0) {
          T p = vs * ys;
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int q = lane8 + 8 * i;
            if (q < qn) p -= vq[i] * sdW[q] + wq[i] * sdV[q];
          }
          p = sum8(p);
          wnew = (in && r >= j) ? tp * p + alpha * vpn : T(0);
          if (in && lane8 == 0) a.Wp[r + (size_t)qn * n] = wnew;
        }
        if (last) continue;
        T acc = T(0);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int q = lane8 + 8 * i;
          const T cw = cW[q], cv = cV[q];
          if (q < qn) {
            acc = fma(vq[i], cw, acc);
            acc = fma(wq[i], cv, acc);
          } else if (q == qn) {
            acc = fma(vpn, cw, acc);
            acc = fma(wnew, cv, acc);
          }
        }
        acc = sum8(acc);
        const T ar = cj - acc;
        if (act && lane8 == 0) colj[r] = ar;
        if (act && r >= j + 2) {
          if (lane8 == 0) sig = fma(ar, ar, sig);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int q = lane8 + 8 * i;
            pdv[i] = fma((q == qn) ? vpn : vq[i], ar, pdv[i]);
            pdw[i] = fma((q == qn) ? wnew : wq[i], ar, pdw[i]);
          }
        }
      }
      if (last) break;
      // per-CTA partials in one pass: the 4 row groups of a warp, then the warps that had rows
      // (w < nused), fixed order (W dots at q, V dots at kPb + q, the squared norm at 2 kPb)
      constexpr int kW = 2 * kPb + 1;
      const int nused = min(kThreads / 32, max(0, (row1 - row0 + 3) / 4));
      if ((t >> 5) < nused) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          pdv[i] += __shfl_xor_sync(0xffffffffu, pdv[i], 8);
          pdv[i] += __shfl_xor_sync(0xffffffffu, pdv[i], 16);
          pdw[i] += __shfl_xor_sync(0xffffffffu, pdw[i], 8);
          pdw[i] += __shfl_xor_sync(0xffffffffu, pdw[i], 16);
        }
        sig += __shfl_xor_sync(0xffffffffu, sig, 8);
        sig += __shfl_xor_sync(0xffffffffu, sig, 16);
      }
      if (lane < 8 && (t >> 5) < nused) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          red[(t >> 5) * kW + lane + 8 * i] = pdw[i];
          red[(t >> 5) * kW + kPb + lane + 8 * i] = pdv[i];
        }
      }
      if (lane == 0 && (t >> 5) < nused) red[(t >> 5) * kW + 2 * kPb] = sig;
      __syncthreads();
      if (t < kW) {
        T sp = T(0);
        for (int w = 0; w < nused; ++w) sp += red[w * kW + t];
        if (t < 2 * kPb)
          a.dpart[(size_t)b * 2 * kPb + t] = sp;
        else
          a.part[b] = sp;
      }
    }
    grid_sync_base(a.bar, nb, a.base, epoch, [] {});
    // ------------------------------------------------------------------------------------- B
    {
      T ssum = (t < G) ? __ldcg(a.part + t) : T(0);
      // the dot this CTA finishes (if any): W(:,q)^T v or V(:,q)^T v
      const bool has_dot = b < 2 * jj;
      const int q = has_dot ? b % jj : 0;
      const bool isV = b >= jj;
      T dp = (has_dot && t < G) ? __ldcg(a.dpart + (size_t)t * 2 * kPb + (isV ? kPb : 0) + q) : T(0);
      T al = T(0), djj = T(0), x1q = T(0);
      if (t == 0) {
        al = __ldcg(colj + j + 1);
        djj = __ldcg(colj + j);
        if (has_dot) x1q = __ldcg((isV ? a.Vp : a.Wp) + (j + 1) + (size_t)q * n);
      }
      // the staged x: raw column entries below j + 1 (x(j+1) is set once the norm is known); all
      // loads issued before the first store
      T raw[kVPer<T>];
#pragma unroll
      for (int k = 0; k < kVPer<T>; ++k) {
        const int kk = t + kThreads * k, r = o + kk;
        raw[k] = (kk < vlen && r >= j + 2 && r < n) ? __ldcg(colj + r) : T(0);
      }
#pragma unroll
      for (int k = 0; k < kVPer<T>; ++k) {
        const int kk = t + kThreads * k;
        if (kk < vlen) vall[kk] = raw[k];
      }
      // the two sums over the CTAs' partials: the warps that hold them (threads t < G), then thread 0
      if ((t >> 5) < (G + 31) / 32) {
        ssum = warp_sum(ssum);
        dp = warp_sum(dp);
        if (lane == 0) {
          sh[t >> 5] = ssum;
          sh[32 + (t >> 5)] = dp;
        }
      }
      __syncthreads();
      if (t == 0) {
        ssum = T(0);
        dp = T(0);
        for (int w = 0; w < (G + 31) / 32; ++w) {
          ssum += sh[w];
          dp += sh[32 + w];
        }
        // dlarfg: beta = -sign(alpha) ||x||, tau = (beta - alpha) / beta, v = x / (alpha - beta)
        T beta, tv, scale;
        if (ssum == T(0)) {
          tv = T(0);
          beta = al;
          scale = T(0);
        } else {
          beta = -copysign(sqrt(al * al + ssum), al);
          tv = (beta - al) / beta;
          scale = T(1) / (al - beta);
        }
        // the tiles multiply x = v / vs: raw column entries, and x(j+1) = alpha - beta
        s_scal[2] = (ssum == T(0)) ? T(1) : scale;
        vall[j + 1 - o] = (ssum == T(0)) ? T(1) : al - beta;
        s_scal[4] = scale;
        if (b == 0) {
          a.d[j] = djj;
          a.e[j] = beta;
          a.tau[j] = tv;
        }
        if (has_dot) a.dots[(isV ? kPb : 0) + q] = scale * dp + x1q;
      }
      __syncthreads();
      const T scale = s_scal[4];
      for (int r = row0 + t; r < row1; r += kThreads) {
        const T v = (r == j + 1) ? T(1) : scale * vall[r - o];
        a.Vp[r + (size_t)jj * n] = v;
        a.V[r + (size_t)j * a.ldv] = v;
      }
      // tile products, each group on its own tiles: thread (row quad i4, column group cg of 8)
      const int i4 = tg & 15, cg = tg >> 4;
      T vacc = T(0);
      for (int kk = 0; kk < Kg; ++kk) {
        int s;
        long long u = 0;
        if (gres) {
          s = kk;
          if (jj == 0) slot_wait(gbar(s), 0, a.bar);
        } else {
          u = (long long)jj * Kg + kk;
          s = (int)(u % ns);
          slot_wait(gbar(s), (uint32_t)((u / ns) & 1), a.bar);
        }
        const T *slot = gslots + (size_t)s * kTile * kTile;
        const int packed = s_tile[g + kGroups * kk];
        const int tr = packed >> 16, tc = packed & 0xffff;
        const bool diag = tr == tc;
        const int r0 = kTile * tr, c0 = kTile * tc;   // offsets into vall
        T vi[4], vc[8], rs[4] = {T(0), T(0), T(0), T(0)}, cs[8];
        lds4(vall + r0 + 4 * i4, vi);
        {
          T v0[4], v1[4];
          lds4(vall + c0 + 8 * cg, v0);
          lds4(vall + c0 + 8 * cg + 4, v1);
#pragma unroll
          for (int e = 0; e < 4; ++e) vc[e] = v0[e], vc[4 + e] = v1[e];
        }
#pragma unroll
        for (int kc = 0; kc < 8; ++kc) {
          const int c = 8 * cg + kc;
          T av[4];
          lds4(slot + c * kTile + 4 * i4, av);
          cs[kc] = T(0);
#pragma unroll
          for (int ri = 0; ri < 4; ++ri) {
            const int r = 4 * i4 + ri;
            const T ar = (!diag || c <= r) ? av[ri] : T(0);   // diagonal tile: lower triangle only
            const T ac = (!diag || c < r) ? av[ri] : T(0);
            rs[ri] = fma(ar, vc[kc], rs[ri]);
            cs[kc] = fma(ac, vi[ri], cs[kc]);
          }
        }
        // column totals over the 64 rows: the 16 lanes of a half warp share the column group
        const T ctot = transpose_sum8_16(cs);
        const int ccol = 8 * cg + ((lane >> 1) & 7);
        // row partials: the two column groups of the warp, then the group's four warps
#pragma unroll
        for (int ri = 0; ri < 4; ++ri) rs[ri] += __shfl_xor_sync(0xffffffffu, rs[ri], 16);
        T *gb = gred + (kk & 1) * (kGroups * kTile + kTile);
        if (lane < 16) {
#pragma unroll
          for (int ri = 0; ri < 4; ++ri) gb[wg * kTile + 4 * i4 + ri] = rs[ri];
        }
        if ((lane & 1) == 0) {
          if (diag) {
            gb[kGroups * kTile + ccol] = ctot;
          } else {
            a.P[((size_t)tc * nt + tr) * kTile + ccol] = ctot;
            vacc = fma(vall[c0 + ccol], ctot, vacc);
          }
        }
        group_sync(g);
        if (!gres && u + ns < glen) gissue((int)((u + ns) % Kg), s);
        if (tg < kTile) {
          T sr = gb[tg] + gb[kTile + tg] + gb[2 * kTile + tg] + gb[3 * kTile + tg];
          if (diag) sr += gb[kGroups * kTile + tg];
          a.P[((size_t)tr * nt + tc) * kTile + tg] = sr;
          vacc = fma(vall[r0 + tg], sr, vacc);
        }
      }
      vacc = warp_sum(vacc);
      if (lane == 0) sh[t >> 5] = vacc;
    }
    // the CTA's partial of v^T A22 v, summed over the warps by thread 0 at the barrier's entry
    grid_sync_base(a.bar, nb, a.base, epoch, [&] {
      T v = T(0);
      for (int w = 0; w < kThreads / 32; ++w) v += sh[w];
      a.vpart[b] = v;
    });
  }
  if (t == 0 && a.status != nullptr && *(volatile int *)&a.bar->err != 0) atomicMax(a.status, (int)kDevIterCap);
}

}  // namespace

template <typename T>
bool panel_resident_plan(int n, T *A, int lda, PanelResidentPlan &p) {
  p = PanelResidentPlan{};
  const int vlen = (n + kTile - 1) / kTile * kTile;
  if (n < 2 || vlen > kThreads * kVPer<T>) return false;
  const bool aligned = ((uintptr_t)A % 16 == 0) && (((size_t)lda * sizeof(T)) % 16 == 0);
  if (aligned && tensor_map_encoder() != nullptr) {
    CUtensorMap *m = reinterpret_cast<CUtensorMap *>(p.tmap);
    const cuuint64_t dims[2] = {(cuuint64_t)n, (cuuint64_t)n};
    const cuuint64_t strides[1] = {(cuuint64_t)lda * sizeof(T)};
    const cuuint32_t box[2] = {kTile, kTile}, es[2] = {1, 1};
    const CUresult r = tensor_map_encoder()(m, sizeof(T) == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                                   (void *)A, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                   CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    p.tma = r == CUDA_SUCCESS;
  }
  const void *kern = p.tma ? (const void *)sytrd_panel_resident_kernel<T, true>
                           : (const void *)sytrd_panel_resident_kernel<T, false>;
  // dynamic shared memory: the device's per-block opt-in limit less the kernel's static part
  int dev = 0, optin = 0, sms = 0;
  cudaFuncAttributes fa{};
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaFuncGetAttributes(&fa, kern) != cudaSuccess)
    return false;
  const size_t budget = (size_t)optin - fa.sharedSizeBytes;
  const size_t fixed = (size_t)(vlen + kRed) * sizeof(T);
  const size_t tile = (size_t)kTile * kTile * sizeof(T);
  if (fixed + (size_t)kGroups * tile > budget) return false;
  p.nslot = (int)std::min<size_t>(kMaxSlots, (budget - fixed) / tile);
  if (g_panel_mode.load() == 2) p.nslot = std::min(p.nslot, 2 * kGroups);
  p.smem = (int)(p.nslot * tile + fixed);
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, p.smem) != cudaSuccess) return false;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, p.smem) != cudaSuccess || per_sm < 1)
    return false;
  p.ctas = sms;   // one CTA per SM
  if (g_panel_mode.load() == 2) p.ctas = std::min(p.ctas, 2 * kPb);
  // tiles of one CTA in the first panel (the largest), bounded by the coordinate table
  const long long nt0 = (n + kTile - 1) / kTile, ntiles0 = nt0 * (nt0 + 1) / 2;
  if (p.ctas < 2 * kPb || p.ctas > kThreads || (ntiles0 + p.ctas - 1) / p.ctas > kMaxK) return false;
  p.ok = true;
  return true;
}

template <typename T>
void panel_resident_launch(cudaStream_t s, const PanelResidentPlan &p, int ctas, T *A, int lda, int n, int p0, int nbp,
                           T *Vp, T *Wp, T *P, T *dots, T *part, T *vpart, T *dpart, T *V, int ldv, T *d, T *e,
                           T *tau, GridBar *bar, unsigned base, int *status) {
  Args<T> a{A, lda, n, p0, nbp, p.nslot, Vp, Wp, P, dots, part, vpart, dpart, V, d, e, tau, ldv, bar, base, status};
  CUtensorMap map;
  std::memcpy(&map, p.tmap, sizeof(map));
  void *args[] = {&map, &a};
  if (p.tma)
    cudaLaunchCooperativeKernel((const void *)sytrd_panel_resident_kernel<T, true>, dim3(ctas), dim3(kThreads), args,
                                (size_t)p.smem, s);
  else
    cudaLaunchCooperativeKernel((const void *)sytrd_panel_resident_kernel<T, false>, dim3(ctas), dim3(kThreads), args,
                                (size_t)p.smem, s);
  count_launch();
}

template bool panel_resident_plan<float>(int, float *, int, PanelResidentPlan &);
template bool panel_resident_plan<double>(int, double *, int, PanelResidentPlan &);
template void panel_resident_launch<float>(cudaStream_t, const PanelResidentPlan &, int, float *, int, int, int, int,
                                           float *, float *, float *, float *, float *, float *, float *, float *, int,
                                           float *, float *, float *, GridBar *, unsigned, int *);
template void panel_resident_launch<double>(cudaStream_t, const PanelResidentPlan &, int, double *, int, int, int, int,
                                            double *, double *, double *, double *, double *, double *, double *,
                                            double *, int, double *, double *, double *, GridBar *, unsigned, int *);

}  // namespace dg
