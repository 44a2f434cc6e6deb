// Symmetric tridiagonal eigensolver by level-synchronous divide and conquer (Cuppen's method with
// Dongarra-Sorensen deflation and the Gu-Eisenstat recomputation of z for orthogonality).
//
// The tridiagonal is torn at every block boundary (T = diag(T1, T2) + |beta| u u^T, u = e_m-1 +
// sign(beta) e_m), leaves are single elements, and each level merges pairs of neighbouring blocks:
//   sort    : merge the two sorted eigenvalue lists, form z = [Q1(last,:), sign Q2(first,:)] / sqrt2
//   deflate : small |z| or close eigenvalue pairs (Givens rotation of the two Q columns)
//   secular : 1 + rho sum w_j^2 / (d_j - lambda) = 0, one warp per root, bracketed two-pole
//             rational iteration with bisection safeguard (bounded iterations, status on cap)
//   zhat    : z_j^2 = prod_i (lambda_i - d_j) / (rho prod_{i != j} (d_i - d_j))
//   vectors : U(:, i) = zhat / (d - lambda_i), normalised; Q_new = Q_nondeflated * U as two GEMMs,
//             one per half of the rows: the surviving columns are grouped by row support (left
//             half only, both halves after a rotation across the halves, right half only), and
//             each half multiplies only the groups that are non-zero in it (half the FLOPs when no
//             rotation crosses the halves)
//   scatter : final ascending order of roots and deflated values, columns placed accordingly.
// This replaces the tridiagonal stage of dsygvd (math/eigensolver.F90:561-660 'D' solvers).
#include <algorithm>
#include <vector>

#include <atomic>

#include "linalg.cuh"

namespace dg {

constexpr int kSecularMaxIter = 100;
constexpr int kSmallMerge = 128;   // merges up to this size use the batched in-CTA product

struct Merge {
  int a, m, b;   // left block [a, m), right block [m, b); m == b means pass-through
  int pad;
};

template <typename T>
struct DcWork {
  T *Ds, *zs, *dl, *w, *tau, *lam, *zh, *rot_cs, *vals;
  int *perm, *ndpos, *dfpos, *org, *rot_cols, *mK, *mRot, *srcinfo;
  // grp[a + k]: column of the surviving pole k in the type-grouped order of the merge product (rows
  // of U, columns of Gs): columns supported on the left half only, then on both halves (a rotation
  // across the halves), then on the right half only; mK1 / mK2 per merge: the first two group ends
  int *grp, *mK1, *mK2;
  T *Gs, *U, *Qtmp, *Qalt;
};

// Scalar-type traits: unit roundoff and the range kept by the exponent-tracked products.
template <typename T> struct Lim;
template <> struct Lim<double> {
  static constexpr double eps = 2.220446049250313e-16, big = 1e150, small = 1e-150;
};
template <> struct Lim<float> {
  static constexpr float eps = 1.1920929e-07f, big = 1e30f, small = 1e-30f;
};
__device__ __forceinline__ double t_frexp(double x, int *e) { return frexp(x, e); }
__device__ __forceinline__ float t_frexp(float x, int *e) { return frexpf(x, e); }
__device__ __forceinline__ double t_ldexp(double x, int e) { return ldexp(x, e); }
__device__ __forceinline__ float t_ldexp(float x, int e) { return ldexpf(x, e); }
__device__ __forceinline__ double t_hypot(double x, double y) { return hypot(x, y); }
__device__ __forceinline__ float t_hypot(float x, float y) { return hypotf(x, y); }

template <typename T>
__device__ __forceinline__ T wsum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <typename T>
__device__ __forceinline__ T wmax(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Tear: d[m-1] -= |e[m-1]|, d[m] -= |e[m-1]| for every block boundary m. Leaves are single
// elements, so every m in 1..n-1 is a boundary and each diagonal entry loses both neighbours'
// couplings (one thread per entry: adjacent boundaries share an entry).
template <typename T>
__global__ void dc_tear_kernel(int n, T *d, const T *e) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T v = d[i];
  if (i > 0) v -= fabs(e[i - 1]);
  if (i < n - 1) v -= fabs(e[i]);
  d[i] = v;
}

template <typename T>
__global__ void dc_identity_kernel(int n, T *Q, int ldq) {
  int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    Q[i + (size_t)j * ldq] = (i == j) ? T(1) : T(0);
}

// K1: merge-sort the two eigenvalue lists and form z.
template <typename T>
__global__ void dc_sort_kernel(const Merge *merges, const T *d, const T *e, const T *Q,
                               int ldq, DcWork<T> W) {
  Merge mg = merges[blockIdx.x];
  if (mg.m == mg.b) return;
  const int a = mg.a, m = mg.m, b = mg.b;
  const int nL = m - a, nR = b - m;
  const T sgn = (e[m - 1] >= T(0)) ? T(1) : T(-1);
  const T is2 = T(0.70710678118654752440);
  for (int i = threadIdx.x; i < nL + nR; i += blockDim.x) {
    T val, zv;
    int pos, blk;
    if (i < nL) {
      val = d[a + i];
      zv = Q[(m - 1) + (size_t)(a + i) * ldq] * is2;
      int lo = 0, hi = nR;  // count right elements < val
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (d[m + mid] < val) lo = mid + 1; else hi = mid;
      }
      pos = i + lo;
      blk = i;
    } else {
      int r = i - nL;
      val = d[m + r];
      zv = sgn * Q[m + (size_t)(m + r) * ldq] * is2;
      int lo = 0, hi = nL;  // count left elements <= val
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (d[a + mid] <= val) lo = mid + 1; else hi = mid;
      }
      pos = r + lo;
      blk = nL + r;
    }
    W.Ds[a + pos] = val;
    W.zs[a + pos] = zv;
    W.perm[a + pos] = blk;
  }
}

// K2: deflation. The scan over the sorted entries is sequential (a rotation changes the z entry and
// the pole the next test reads), so one thread runs it after a parallel max reduction. Scan: an
// entry with negligible rho |z_j| deflates; otherwise, against the previous surviving entry, a
// rotation that zeroes z_prev deflates the pair when |(d_j - d_prev) c s| is negligible. F is the
// flag type (1 = deflated); the rotations go to W.rot_cols / W.rot_cs at the merge's offset a. sup
// tracks the row support of each entry's column (1 left half, 2 right half, 3 both after a rotation
// across the halves); the first nL of the merge's N original columns are the left half's.
// Group of a surviving column by its row support: 0 left half only, 1 both halves, 2 right half only.
__device__ __forceinline__ int dc_sup_type(int sup) { return sup == 1 ? 0 : (sup == 3 ? 1 : 2); }

template <typename T, typename F, typename S>
__device__ int dc_deflate_scan(int N, int nL, int a, T *Ds, T *zs, const int *perm, F *flag, S *sup, T rho2, T mz,
                               T tol, const DcWork<T> &W) {
  int nrot = 0;
  for (int j = 0; j < N; ++j) {
    flag[j] = 0;
    sup[j] = (perm[j] < nL) ? 1 : 2;   // row support of the entry's column: 1 left half, 2 right half
  }
  if (rho2 * mz <= tol) {
    for (int j = 0; j < N; ++j) flag[j] = 1;
    return 0;
  }
  int prev = -1;
  for (int j = 0; j < N; ++j) {
    if (rho2 * fabs(zs[j]) <= tol) {
      flag[j] = 1;
      continue;
    }
    if (prev >= 0) {
      T s = zs[prev], c = zs[j];
      T t = t_hypot(c, s);
      T tdiff = Ds[j] - Ds[prev];
      c /= t;
      s = -s / t;
      if (fabs(tdiff * c * s) <= tol) {
        zs[j] = t;
        zs[prev] = T(0);
        W.rot_cols[2 * (a + nrot)] = a + perm[prev];
        W.rot_cols[2 * (a + nrot) + 1] = a + perm[j];
        W.rot_cs[2 * (a + nrot)] = c;
        W.rot_cs[2 * (a + nrot) + 1] = s;
        ++nrot;
        T tt = Ds[prev] * c * c + Ds[j] * s * s;
        Ds[j] = Ds[prev] * s * s + Ds[j] * c * c;
        Ds[prev] = tt;
        flag[prev] = 1;
        sup[j] = sup[j] | sup[prev];
      }
    }
    prev = j;
  }
  return nrot;
}

// One CTA per merge. A merge of at most stage_n entries is staged in dynamic shared memory (its
// sorted poles, z entries, origins, flags and supports: N (2 sizeof(T) + 6) bytes), so each step of the scan
// costs shared-memory latency instead of global round trips, and the compaction (non-deflated
// positions -> ndpos with their poles and z entries in dl / w, deflated positions -> dfpos, both in
// order; the support type of each survivor, 0 left / 1 both / 2 right, to grp) is a CTA-wide prefix
// sum; the staged poles and z entries are written back. A larger merge runs the scan and the
// compaction in global memory by one thread.
template <typename T>
__global__ void __launch_bounds__(256) dc_deflate_kernel(const Merge *merges, const T *e, DcWork<T> W, int stage_n) {
  extern __shared__ __align__(16) unsigned char dc_dsm[];
  const int mi = blockIdx.x;
  Merge mg = merges[mi];
  if (mg.m == mg.b) {
    if (threadIdx.x == 0) { W.mK[mi] = 0; W.mRot[mi] = 0; }
    return;
  }
  const int a = mg.a, N = mg.b - mg.a;
  const int t = threadIdx.x, nt = blockDim.x, lane = t & 31, wid = t >> 5;
  const bool staged = N <= stage_n;
  __shared__ T smax[2][32];
  __shared__ int s_scan[32];
  __shared__ int s_nrot;
  T md = T(0), mz = T(0);
  for (int i = t; i < N; i += nt) {
    md = fmax(md, fabs(W.Ds[a + i]));
    mz = fmax(mz, fabs(W.zs[a + i]));
  }
  md = wmax(md);
  mz = wmax(mz);
  if (lane == 0) { smax[0][wid] = md; smax[1][wid] = mz; }
  T *sD = reinterpret_cast<T *>(dc_dsm), *sZ = sD + N;
  int *sP = reinterpret_cast<int *>(sZ + N);
  unsigned char *sF = reinterpret_cast<unsigned char *>(sP + N), *sS = sF + N;
  if (staged) {
    for (int i = t; i < N; i += nt) {
      sD[i] = W.Ds[a + i];
      sZ[i] = W.zs[a + i];
      sP[i] = W.perm[a + i];
    }
  }
  __syncthreads();
  if (t == 0) {
    for (int k = 1; k < (nt >> 5); ++k) {
      md = fmax(md, smax[0][k]);
      mz = fmax(mz, smax[1][k]);
    }
    md = fmax(md, smax[0][0]);
    mz = fmax(mz, smax[1][0]);
    const T rho2 = T(2) * fabs(e[mg.m - 1]);
    const T tol = T(8) * Lim<T>::eps * fmax(md, mz);
    const int nL = mg.m - mg.a;
    if (staged) {
      s_nrot = dc_deflate_scan(N, nL, a, sD, sZ, sP, sF, sS, rho2, mz, tol, W);
    } else {
      // flags kept in dfpos and supports in grp temporarily; the sequential compaction overwrites both
      // in order (dfpos[q] and grp[q] are written only after entry j >= q has been read)
      T *Ds = W.Ds + a, *zs = W.zs + a;
      int *flag = W.dfpos + a, *sup = W.grp + a;
      const int nrot = dc_deflate_scan(N, nL, a, Ds, zs, W.perm + a, flag, sup, rho2, mz, tol, W);
      int K = 0, nD = 0;
      for (int j = 0; j < N; ++j) {
        if (!flag[j]) {
          const int sj = sup[j];
          W.ndpos[a + K] = j;
          W.dl[a + K] = Ds[j];
          W.w[a + K] = zs[j];
          W.grp[a + K] = dc_sup_type(sj);
          ++K;
        } else {
          flag[nD] = j;
          ++nD;
        }
      }
      W.mK[mi] = K;
      W.mRot[mi] = nrot;
    }
  }
  if (!staged) return;
  __syncthreads();
  // compaction: thread t takes the contiguous chunk [j0, j1); exclusive prefix sum of the surviving
  // counts over the threads
  const int C = (N + nt - 1) / nt;
  const int j0 = min(N, t * C), j1 = min(N, j0 + C);
  int cnt = 0;
  for (int j = j0; j < j1; ++j) cnt += sF[j] ? 0 : 1;
  int inc = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += v;
  }
  if (lane == 31) s_scan[wid] = inc;
  __syncthreads();
  if (t == 0) {
    int run = 0;
    for (int w = 0; w < (nt >> 5); ++w) {
      const int v = s_scan[w];
      s_scan[w] = run;
      run += v;
    }
    W.mK[mi] = run;
    W.mRot[mi] = s_nrot;
  }
  __syncthreads();
  int K = s_scan[wid] + inc - cnt;   // surviving entries before j0
  int nD = j0 - K;                   // deflated entries before j0
  for (int j = j0; j < j1; ++j) {
    if (!sF[j]) {
      W.ndpos[a + K] = j;
      W.dl[a + K] = sD[j];
      W.w[a + K] = sZ[j];
      W.grp[a + K] = dc_sup_type(sS[j]);
      ++K;
    } else {
      W.dfpos[a + nD] = j;
      ++nD;
    }
  }
  for (int i = t; i < N; i += nt) {
    W.Ds[a + i] = sD[i];
    W.zs[a + i] = sZ[i];
  }
}

// Largest merge staged by dc_deflate_kernel and its dynamic shared memory (bytes) for a level whose
// largest block has max_block entries: the merge fits below kDcStageBytes or nothing is staged.
constexpr int kDcStageBytes = 160 * 1024;
std::atomic<int> g_dc_stage{1};
template <typename T>
static int dc_stage_n(int max_block) {
  if (!g_dc_stage.load(std::memory_order_relaxed)) return 0;
  return (size_t)max_block * (2 * sizeof(T) + 6) <= (size_t)kDcStageBytes ? max_block : 0;
}
template <typename T>
static size_t dc_stage_bytes(int stage_n) {
  return (size_t)stage_n * (2 * sizeof(T) + 6);
}

// K2b: positions of the surviving poles in the type-grouped order of the merge product (stable within
// each group), from the types the deflation left in grp; one CTA per merge, prefix sums of the three
// counts over contiguous chunks. mK1 / mK2 receive the ends of the first two groups.
template <typename T>
__global__ void __launch_bounds__(256) dc_group_kernel(const Merge *merges, DcWork<T> W) {
  const int mi = blockIdx.x;
  Merge mg = merges[mi];
  if (mg.m == mg.b) return;
  const int a = mg.a, K = W.mK[mi];
  const int t = threadIdx.x, nt = blockDim.x, lane = t & 31, wid = t >> 5, nw = nt >> 5;
  __shared__ int s_c[3][33];
  const int C = (K + nt - 1) / nt;
  const int k0 = min(K, t * C), k1 = min(K, k0 + C);
  int c0 = 0, c1 = 0, c2 = 0;
  for (int k = k0; k < k1; ++k) {
    const int ty = W.grp[a + k];
    c0 += (ty == 0);
    c1 += (ty == 1);
    c2 += (ty == 2);
  }
  int i0 = c0, i1 = c1, i2 = c2;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v0 = __shfl_up_sync(0xffffffffu, i0, o);
    const int v1 = __shfl_up_sync(0xffffffffu, i1, o);
    const int v2 = __shfl_up_sync(0xffffffffu, i2, o);
    if (lane >= o) {
      i0 += v0;
      i1 += v1;
      i2 += v2;
    }
  }
  if (lane == 31) {
    s_c[0][wid] = i0;
    s_c[1][wid] = i1;
    s_c[2][wid] = i2;
  }
  __syncthreads();
  if (t == 0) {
    for (int q = 0; q < 3; ++q) {
      int run = 0;
      for (int w = 0; w < nw; ++w) {
        const int v = s_c[q][w];
        s_c[q][w] = run;
        run += v;
      }
      s_c[q][32] = run;
    }
    W.mK1[mi] = s_c[0][32];
    W.mK2[mi] = s_c[0][32] + s_c[1][32];
  }
  __syncthreads();
  int p0 = s_c[0][wid] + i0 - c0;
  int p1 = s_c[0][32] + s_c[1][wid] + i1 - c1;
  int p2 = s_c[0][32] + s_c[1][32] + s_c[2][wid] + i2 - c2;
  for (int k = k0; k < k1; ++k) {
    const int ty = W.grp[a + k];
    W.grp[a + k] = (ty == 0) ? p0++ : ((ty == 1) ? p1++ : p2++);
  }
}

// K3: apply the recorded rotations to the Q columns (each thread owns a row of the block).
template <typename T>
__global__ void dc_rotate_kernel(const Merge *merges, T *Q, int ldq, DcWork<T> W) {
  const int mi = blockIdx.x;
  Merge mg = merges[mi];
  if (mg.m == mg.b) return;
  const int nrot = W.mRot[mi];
  if (nrot == 0) return;
  int row = mg.a + blockIdx.y * blockDim.x + threadIdx.x;
  if (row >= mg.b) return;
  for (int k = 0; k < nrot; ++k) {
    int cp = W.rot_cols[2 * (mg.a + k)], cj = W.rot_cols[2 * (mg.a + k) + 1];
    T c = W.rot_cs[2 * (mg.a + k)], s = W.rot_cs[2 * (mg.a + k) + 1];
    T x = Q[row + (size_t)cp * ldq], y = Q[row + (size_t)cj * ldq];
    Q[row + (size_t)cp * ldq] = c * x + s * y;
    Q[row + (size_t)cj * ldq] = c * y - s * x;
  }
}

// K4: secular equation, one warp per root.
template <typename T>
__global__ void dc_secular_kernel(int n, const Merge *merges, const int *pos_merge, const T *e,
                                  DcWork<T> W, int *status) {
  const int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (g >= n) return;
  const int mi = pos_merge[g];
  if (mi < 0) return;
  Merge mg = merges[mi];
  const int a = mg.a;
  const int K = W.mK[mi];
  const int i = g - a;
  if (i >= K) return;
  const T rho = T(2) * fabs(e[mg.m - 1]);
  const T *dl = W.dl + a, *w = W.w + a;
  int org;
  T lo, hi, tau;
  if (i < K - 1) {
    T mid = T(0.5) * (dl[i + 1] - dl[i]);
    T s = T(0);
    for (int j = lane; j < K; j += 32) s += w[j] * w[j] / ((dl[j] - dl[i]) - mid);
    T f = T(1) + rho * wsum(s);
    if (f > T(0)) { org = i; lo = T(0); hi = mid; }
    else { org = i + 1; lo = -mid; hi = T(0); }
  } else {
    T s = T(0);
    for (int j = lane; j < K; j += 32) s += w[j] * w[j];
    org = K - 1;
    lo = T(0);
    hi = rho * wsum(s);
  }
  tau = T(0.5) * (lo + hi);
  const T dorg = dl[org];
  bool conv = false;
  for (int it = 0; it < kSecularMaxIter; ++it) {
    T sf = T(0), sp = T(0), sq = T(0), sa = T(0);
    for (int j = lane; j < K; j += 32) {
      T dd = (dl[j] - dorg) - tau;
      T t = w[j] * w[j] / dd;
      sf += t;
      sa += fabs(t);
      if (j <= i) sp += t / dd; else sq += t / dd;
    }
    T f = T(1) + rho * wsum(sf);
    T psip = rho * wsum(sp);
    T phip = rho * wsum(sq);
    // rounding-error bound of the evaluated f (cf. the ERRETM test of LAPACK's dlaed4)
    T ferr = Lim<T>::eps * (T(8) * (T(1) + rho * wsum(sa)) + fabs(tau) * (psip + phip));
    if (f > T(0)) hi = tau; else lo = tau;
    if (fabs(f) <= ferr) { conv = true; break; }
    T nt;
    if (i < K - 1) {
      T dlo = (dl[i] - dorg) - tau, dhi = (dl[i + 1] - dorg) - tau;
      T A = psip * dlo * dlo, B = phip * dhi * dhi;
      T c = f - A / dlo - B / dhi;
      T A2 = c, B2 = -(c * (dlo + dhi) + A + B), C2 = c * dlo * dhi + A * dhi + B * dlo;
      T st;
      if (A2 == T(0)) {
        st = (B2 != T(0)) ? -C2 / B2 : 0.0;
      } else {
        T disc = sqrt(fmax(B2 * B2 - T(4) * A2 * C2, T(0)));
        T s1, s2;
        if (B2 <= T(0)) {
          T den = -B2 + disc;
          s1 = den / (T(2) * A2);
          s2 = (den != T(0)) ? T(2) * C2 / den : s1;
        } else {
          T den = -B2 - disc;
          s1 = den / (T(2) * A2);
          s2 = T(2) * C2 / den;
        }
        st = (s2 > dlo && s2 < dhi) ? s2 : s1;
      }
      nt = tau + st;
    } else {
      T dlo = (dl[K - 1] - dorg) - tau;
      T A = psip * dlo * dlo;
      T c = f - A / dlo;
      nt = tau + ((c != T(0)) ? dlo + A / c : 0.0);
    }
    if (!(nt > lo && nt < hi)) nt = T(0.5) * (lo + hi);
    if (nt == tau || fabs(hi - lo) <= T(2) * Lim<T>::eps * fmax(fabs(lo), fabs(hi))) {
      tau = nt;
      conv = true;
      break;
    }
    tau = nt;
  }
  if (lane == 0) {
    if (!conv) atomicExch(status, kDevIterCap);
    W.org[a + i] = org;
    W.tau[a + i] = tau;
    W.lam[a + i] = dorg + tau;
  }
}

// K5: Gu-Eisenstat zhat, one warp per j; product of O(1) ratios with exponent tracking.
template <typename T>
__global__ void dc_zhat_kernel(int n, const Merge *merges, const int *pos_merge, const T *e, DcWork<T> W) {
  const int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (g >= n) return;
  const int mi = pos_merge[g];
  if (mi < 0) return;
  Merge mg = merges[mi];
  const int a = mg.a;
  const int K = W.mK[mi];
  const int j = g - a;
  if (j >= K) return;
  const T rho = T(2) * fabs(e[mg.m - 1]);
  const T *dl = W.dl + a;
  const T dj = dl[j];
  T p = 1.0;
  int ex = 0;
  for (int i = lane; i < K; i += 32) {
    T num = (dl[W.org[a + i]] - dj) + W.tau[a + i];
    T r = (i == j) ? num / rho : num / (dl[i] - dj);
    p *= r;
    T ap = fabs(p);
    if (ap > Lim<T>::big || (ap < Lim<T>::small && ap > T(0))) {
      int k;
      p = t_frexp(p, &k);
      ex += k;
    }
  }
  // combine lane products
  for (int o = 16; o > 0; o >>= 1) {
    T po = __shfl_xor_sync(0xffffffffu, p, o);
    int eo = __shfl_xor_sync(0xffffffffu, ex, o);
    p *= po;
    ex += eo;
    int k;
    p = t_frexp(p, &k);
    ex += k;
  }
  if (lane == 0) {
    T val = t_ldexp(p, ex);
    T z = sqrt(fmax(val, T(0)));
    W.zh[a + j] = copysign(z, W.w[a + j]);
  }
}

// K6: eigenvector matrix of the rank-one problem, one warp per column i; U rows [0,K) at column a+i,
// row grp[a + t] for pole t (the type-grouped order of the merge product).
template <typename T>
__global__ void dc_build_u_kernel(int n, const Merge *merges, const int *pos_merge, DcWork<T> W, int ldu) {
  const int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (g >= n) return;
  const int mi = pos_merge[g];
  if (mi < 0) return;
  Merge mg = merges[mi];
  const int a = mg.a;
  const int K = W.mK[mi];
  const int i = g - a;
  if (i >= K) return;
  const T *dl = W.dl + a;
  const T dorg = dl[W.org[a + i]];
  const T tau = W.tau[a + i];
  T *u = W.U + (size_t)(a + i) * ldu;
  T s = T(0);
  for (int t = lane; t < K; t += 32) {
    T v = W.zh[a + t] / ((dl[t] - dorg) - tau);
    u[W.grp[a + t]] = v;
    s += v * v;
  }
  T inv = T(1) / sqrt(wsum(s));
  for (int t = lane; t < K; t += 32) u[t] *= inv;
}

// K7: gather the non-deflated Q columns (rows [a,b)) into Gs at columns a .. a+K-1, pole t at column
// a + grp[a + t].
template <typename T>
__global__ void dc_gather_kernel(int n, const Merge *merges, const int *pos_merge, const T *Q, int ldq,
                                 DcWork<T> W, int ldg) {
  const int g = blockIdx.x;
  const int mi = pos_merge[g];
  if (mi < 0) return;
  Merge mg = merges[mi];
  const int a = mg.a;
  const int K = W.mK[mi];
  const int t = g - a;
  if (t >= K) return;
  const int src = a + W.perm[a + W.ndpos[a + t]];
  const size_t dst = (size_t)(a + W.grp[a + t]) * ldg;
  for (int r = mg.a + threadIdx.x; r < mg.b; r += blockDim.x) W.Gs[r + dst] = Q[r + (size_t)src * ldq];
}

// K8 (small merges): Qtmp[a:b, a:a+K] = Gs[a:b, a:a+K] * U[0:K, a:a+K] inside one CTA.
template <typename T>
__global__ void dc_small_gemm_kernel(const Merge *merges, DcWork<T> W, int ld) {
  Merge mg = merges[blockIdx.x];
  if (mg.m == mg.b) return;
  const int K = W.mK[blockIdx.x];
  const int a = mg.a, N = mg.b - mg.a;
  for (int idx = threadIdx.x; idx < N * K; idx += blockDim.x) {
    int r = idx % N, c = idx / N;
    T s = T(0);
    const T *g = W.Gs + (a + r) + (size_t)a * ld;
    const T *u = W.U + (size_t)(a + c) * ld;
    for (int t = 0; t < K; ++t) s = fma(g[(size_t)t * ld], u[t], s);
    W.Qtmp[(a + r) + (size_t)(a + c) * ld] = s;
  }
}

// K9: final ascending order (rank in the union of roots and deflated values, ties by index).
template <typename T>
__global__ void dc_rank_kernel(const Merge *merges, T *d, DcWork<T> W) {
  const int mi = blockIdx.x;
  Merge mg = merges[mi];
  const int a = mg.a, N = mg.b - mg.a;
  int e0 = blockIdx.y * blockDim.x + threadIdx.x;
  if (e0 >= N) return;
  if (mg.m == mg.b) {  // pass-through block: identity mapping
    W.srcinfo[a + e0] = a + e0;
    W.vals[a + e0] = d[a + e0];
    return;
  }
  const int K = W.mK[mi];
  auto value = [&](int k) -> T {
    return (k < K) ? W.lam[a + k] : W.Ds[a + W.dfpos[a + (k - K)]];
  };
  T v = value(e0);
  int rank = 0;
  for (int k = 0; k < N; ++k) {
    T u = value(k);
    if (u < v || (u == v && k < e0)) ++rank;
  }
  W.vals[a + rank] = v;
  // source column: >= 0 -> column of Q (deflated); < 0 -> -(1 + column of Qtmp)
  W.srcinfo[a + rank] = (e0 < K) ? -(1 + a + e0) : (a + W.perm[a + W.dfpos[a + (e0 - K)]]);
}

// K10: scatter the columns into the output buffer and the values into d.
template <typename T>
__global__ void dc_scatter_kernel(int n, const int *pos_merge_all, const Merge *merges, const T *Q,
                                  int ldq, T *Qout, T *d, DcWork<T> W, int ldt) {
  const int g = blockIdx.x;
  const int mi = pos_merge_all[g];
  Merge mg = merges[mi];
  int src = W.srcinfo[g];
  const T *col = (src >= 0) ? Q + (size_t)src * ldq : W.Qtmp + (size_t)(-src - 1) * ldt;
  for (int r = mg.a + threadIdx.x; r < mg.b; r += blockDim.x) Qout[r + (size_t)g * ldq] = col[r];
  if (threadIdx.x == 0) d[g] = W.vals[g];
}

// ------------------------------------------------------------------------------------- host side
struct DcLevel {
  std::vector<Merge> merges;
  std::vector<int> pos_merge;      // merge index for positions inside real merges, -1 otherwise
  std::vector<int> pos_merge_all;  // merge index (including pass-through) for every position
  int max_block = 0;
};

static std::vector<DcLevel> plan_levels(int n, std::vector<int> &bounds) {
  std::vector<std::pair<int, int>> cur;
  for (int i = 0; i < n; ++i) cur.push_back({i, i + 1});
  std::vector<DcLevel> levels;
  while (cur.size() > 1) {
    DcLevel L;
    std::vector<std::pair<int, int>> nxt;
    for (size_t k = 0; k < cur.size(); k += 2) {
      if (k + 1 < cur.size()) {
        L.merges.push_back({cur[k].first, cur[k].second, cur[k + 1].second, 0});
        bounds.push_back(cur[k].second);
        nxt.push_back({cur[k].first, cur[k + 1].second});
      } else {
        L.merges.push_back({cur[k].first, cur[k].second, cur[k].second, 0});
        nxt.push_back(cur[k]);
      }
    }
    L.pos_merge.assign(n, -1);
    L.pos_merge_all.assign(n, -1);
    for (size_t mi = 0; mi < L.merges.size(); ++mi) {
      const Merge &mg = L.merges[mi];
      for (int p = mg.a; p < mg.b; ++p) {
        L.pos_merge_all[p] = (int)mi;
        if (mg.m != mg.b) L.pos_merge[p] = (int)mi;
      }
      L.max_block = std::max(L.max_block, mg.b - mg.a);
    }
    levels.push_back(std::move(L));
    cur.swap(nxt);
  }
  return levels;
}

size_t stedc_work_size(int n) {
  // 9 vectors of n, rotations (2n), 4 matrices n x n
  return (size_t)n * 9 + 2 * (size_t)n + 4 * (size_t)n * n + 64;
}
size_t stedc_iwork_size(int n) {
  int levels = 0;
  while ((1LL << levels) < n) ++levels;
  // 13 n index vectors + plan metadata (bounds n, merges 4 n, two position maps per level)
  return (size_t)n * (13 + 1 + 4 + 2 * (size_t)(levels + 1)) + 64;
}

// C (rows x cols) = A (rows x kd) B (kd x cols), all with leading dimension ld; C = 0 when kd = 0.
template <typename T>
static void merge_product(cudaStream_t s, int rows, int cols, int kd, const T *A, const T *B, T *C, int ld) {
  if (rows <= 0 || cols <= 0) return;
  if (kd <= 0) {
    cudaMemset2DAsync(C, (size_t)ld * sizeof(T), 0, (size_t)rows * sizeof(T), (size_t)cols, s);
    return;
  }
  gemm<T>(s, 'N', 'N', rows, cols, kd, T(1), A, ld, B, ld, T(0), C, ld);
}

template <typename T>
int stedc(cudaStream_t s, int n, T *d, T *e, T *Q, int ldq, T *work, int *iwork, int *status_dev) {
  if (n <= 0) return 0;
  if (ldq != n) return -1;  // the workspace layout assumes a square, tightly packed Q
  dim3 gi(ceil_div(n, 256), n);
  dc_identity_kernel<T><<<gi, 256, 0, s>>>(n, Q, ldq);
  count_launch();
  if (n == 1) return 0;
  std::vector<int> bounds;
  std::vector<DcLevel> levels = plan_levels(n, bounds);

  DcWork<T> W;
  T *p = work;
  W.Ds = p; p += n; W.zs = p; p += n; W.dl = p; p += n; W.w = p; p += n; W.tau = p; p += n;
  W.lam = p; p += n; W.zh = p; p += n; W.vals = p; p += n; p += n;
  W.rot_cs = p; p += 2 * (size_t)n;
  W.Gs = p; p += (size_t)n * n; W.U = p; p += (size_t)n * n; W.Qtmp = p; p += (size_t)n * n;
  W.Qalt = p; p += (size_t)n * n;
  int *ip = iwork;
  W.perm = ip; ip += n; W.ndpos = ip; ip += n; W.dfpos = ip; ip += n; W.org = ip; ip += n;
  W.srcinfo = ip; ip += n; W.mK = ip; ip += n; W.mRot = ip; ip += n; ip += n;
  W.grp = ip; ip += n; W.mK1 = ip; ip += n; W.mK2 = ip; ip += n;
  W.rot_cols = ip; ip += 2 * (size_t)n;
  int *dev_meta = ip;  // bounds + per-level merges and position maps (uploaded below)

  // upload the plan: bounds, then per level (merges, pos_merge, pos_merge_all)
  std::vector<int> meta(bounds.begin(), bounds.end());
  std::vector<size_t> off_merge, off_pm, off_pma;
  for (auto &L : levels) {
    off_merge.push_back(meta.size());
    for (auto &mg : L.merges) { meta.push_back(mg.a); meta.push_back(mg.m); meta.push_back(mg.b); meta.push_back(0); }
    off_pm.push_back(meta.size());
    meta.insert(meta.end(), L.pos_merge.begin(), L.pos_merge.end());
    off_pma.push_back(meta.size());
    meta.insert(meta.end(), L.pos_merge_all.begin(), L.pos_merge_all.end());
  }
  // the metadata lives in a dedicated device allocation owned by the caller's iwork tail
  cudaMemcpyAsync(dev_meta, meta.data(), meta.size() * sizeof(int), cudaMemcpyHostToDevice, s);

  dc_tear_kernel<T><<<ceil_div(n, 256), 256, 0, s>>>(n, d, e);
  count_launch();
  // The merge at level L reads whole blocks [a,b)^2 whose off-diagonal sub-blocks must be zero;
  // the scatter only writes inside the current blocks, so the second buffer starts zeroed.
  cudaMemsetAsync(W.Qalt, 0, sizeof(T) * (size_t)n * n, s);

  T *Qin = Q, *Qout = W.Qalt;
  std::vector<int> hK;
  for (size_t li = 0; li < levels.size(); ++li) {
    DcLevel &L = levels[li];
    const Merge *dm = reinterpret_cast<const Merge *>(dev_meta + off_merge[li]);
    const int *pm = dev_meta + off_pm[li];
    const int *pma = dev_meta + off_pma[li];
    int nm = (int)L.merges.size();
    dc_sort_kernel<T><<<nm, 256, 0, s>>>(dm, d, e, Qin, ldq, W);
    {
      ensure_dyn_smem((const void *)dc_deflate_kernel<T>, kDcStageBytes);
      const int sn = dc_stage_n<T>(L.max_block);
      dc_deflate_kernel<T><<<nm, 256, dc_stage_bytes<T>(sn), s>>>(dm, e, W, sn);
    }
    dc_group_kernel<T><<<nm, 256, 0, s>>>(dm, W);
    count_launch();
    dim3 gr(nm, ceil_div(L.max_block, 256));
    dc_rotate_kernel<T><<<gr, 256, 0, s>>>(dm, Qin, ldq, W);
    int warps_blocks = ceil_div((long long)n * 32, 256);
    dc_secular_kernel<T><<<warps_blocks, 256, 0, s>>>(n, dm, pm, e, W, status_dev);
    dc_zhat_kernel<T><<<warps_blocks, 256, 0, s>>>(n, dm, pm, e, W);
    dc_build_u_kernel<T><<<warps_blocks, 256, 0, s>>>(n, dm, pm, W, n);
    dc_gather_kernel<T><<<n, 128, 0, s>>>(n, dm, pm, Qin, ldq, W, n);
    count_launch(7);
    if (L.max_block <= kSmallMerge) {
      dc_small_gemm_kernel<T><<<nm, 256, 0, s>>>(dm, W, n);
      count_launch();
    } else {
      hK.resize(3 * (size_t)nm);
      cudaMemcpyAsync(hK.data(), W.mK, nm * sizeof(int), cudaMemcpyDeviceToHost, s);
      cudaMemcpyAsync(hK.data() + nm, W.mK1, nm * sizeof(int), cudaMemcpyDeviceToHost, s);
      cudaMemcpyAsync(hK.data() + 2 * (size_t)nm, W.mK2, nm * sizeof(int), cudaMemcpyDeviceToHost, s);
      cudaStreamSynchronize(s);
      for (int k = 0; k < nm; ++k) {
        const Merge &mg = L.merges[k];
        if (mg.m == mg.b || hK[k] == 0) continue;
        const int a = mg.a, m = mg.m, b = mg.b, K = hK[k], K1 = hK[nm + k], K2 = hK[2 * (size_t)nm + k];
        // Qtmp = Gs U, split by rows: the left rows see only the columns supported there (groups
        // [0, K2)), the right rows only [K1, K); the other columns are zero in those rows
        merge_product<T>(s, m - a, K, K2, W.Gs + a + (size_t)a * n, W.U + (size_t)a * n,
                         W.Qtmp + a + (size_t)a * n, n);
        merge_product<T>(s, b - m, K, K - K1, W.Gs + m + (size_t)(a + K1) * n, W.U + K1 + (size_t)a * n,
                         W.Qtmp + m + (size_t)a * n, n);
      }
    }
    dim3 grk(nm, ceil_div(L.max_block, 256));
    dc_rank_kernel<T><<<grk, 256, 0, s>>>(dm, d, W);
    dc_scatter_kernel<T><<<n, 128, 0, s>>>(n, pma, dm, Qin, ldq, Qout, d, W, n);
    count_launch(2);
    std::swap(Qin, Qout);
  }
  if (Qin != Q) {
    cudaMemcpyAsync(Q, Qin, sizeof(T) * (size_t)n * n, cudaMemcpyDeviceToDevice, s);
  }
  return 0;
}

template int stedc<double>(cudaStream_t, int, double *, double *, double *, int, double *, int *, int *);
template int stedc<float>(cudaStream_t, int, float *, float *, float *, int, float *, int *, int *);

// ------------------------------------------------------------------------------------- no-alloc
// Allocation-free variant for callers that cannot allocate device memory (a solver step running
// inside CUDA stream capture, where cudaMalloc is not permitted; a host program whose device memory
// is owned by another allocator or pool; an MD loop that must not trigger the device-wide
// synchronisation cudaMalloc implies). All scratch lives in one file-scope device array sized for
// n <= kNoAllocMaxN, and the level plan is built on the device, so no host or device memory is
// allocated per call.
constexpr int kNoAllocMaxN = 256;
constexpr int kNoAllocMaxLevels = 8;                   // ceil(log2 256)
constexpr size_t kNoAllocWork = 9 * 256 + 2 * 256 + 4 * 256 * 256 + 64;      // doubles
constexpr size_t kNoAllocPlan = 4 * 256 + 2 * 256 * kNoAllocMaxLevels + 64;  // ints
constexpr size_t kNoAllocIwork = 13 * 256 + kNoAllocPlan + 64;                // ints
constexpr size_t kNoAllocDoubles = kNoAllocWork + (kNoAllocIwork + 1) / 2 + 32;

// ~2.2 MB per device, held by every GPU that loads the library until process exit. Shared by all
// calls: it keeps the previous call's contents, and calls that overlap on the GPU race on it.
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

struct DcPlanOffsets {
  int nlev;
  int nm[kNoAllocMaxLevels + 1];
  int off_merge[kNoAllocMaxLevels + 1], off_pm[kNoAllocMaxLevels + 1], off_pma[kNoAllocMaxLevels + 1];
};

// The pairwise merge tree of single-element leaves has blocks of 2^L elements at level L
// (the last one truncated; a block without a right half passes through unchanged).
__global__ void dc_plan_kernel(int n, DcPlanOffsets P, int *meta) {
  for (int L = 1; L <= P.nlev; ++L) {
    const int size = 1 << L;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < n; g += gridDim.x * blockDim.x) {
      int mi = g >> L;
      int a = mi << L;
      int b = min(a + size, n);
      int m = min(a + (size >> 1), b);
      meta[P.off_pma[L] + g] = mi;
      meta[P.off_pm[L] + g] = (m == b) ? -1 : mi;
      if (g == a) {
        int *mg = meta + P.off_merge[L] + 4 * mi;
        mg[0] = a; mg[1] = m; mg[2] = b; mg[3] = 0;
      }
    }
  }
}

static int stedc_noalloc_impl(cudaStream_t s, int n, double *d, const double *e_in, double *Q, double *scratch) {
  double *e = const_cast<double *>(e_in);  // read only
  DcWork<double> W;
  double *p = scratch;
  W.Ds = p; p += n; W.zs = p; p += n; W.dl = p; p += n; W.w = p; p += n; W.tau = p; p += n;
  W.lam = p; p += n; W.zh = p; p += n; W.vals = p; p += n; p += n;
  W.rot_cs = p; p += 2 * (size_t)n;
  W.Gs = p; p += (size_t)n * n; W.U = p; p += (size_t)n * n; W.Qtmp = p; p += (size_t)n * n;
  W.Qalt = p;
  int *ip = reinterpret_cast<int *>(scratch + kNoAllocWork);
  int *status = ip; ip += 32;
  W.perm = ip; ip += n; W.ndpos = ip; ip += n; W.dfpos = ip; ip += n; W.org = ip; ip += n;
  W.srcinfo = ip; ip += n; W.mK = ip; ip += n; W.mRot = ip; ip += n; ip += n;
  W.grp = ip; ip += n; W.mK1 = ip; ip += n; W.mK2 = ip; ip += n;
  W.rot_cols = ip; ip += 2 * (size_t)n;
  int *meta = ip;

  DcPlanOffsets P{};
  int nlev = 0;
  while ((1 << nlev) < n) ++nlev;
  P.nlev = nlev;
  int off = 0;
  for (int L = 1; L <= nlev; ++L) {
    P.nm[L] = (n + (1 << L) - 1) >> L;
    P.off_merge[L] = off; off += 4 * P.nm[L];
    P.off_pm[L] = off; off += n;
    P.off_pma[L] = off; off += n;
  }
  cudaMemsetAsync(status, 0, sizeof(int), s);
  dim3 gi(ceil_div(n, 256), n);
  dc_identity_kernel<double><<<gi, 256, 0, s>>>(n, Q, n);
  count_launch();
  if (n == 1) return 0;
  dc_plan_kernel<<<1, 256, 0, s>>>(n, P, meta);
  dc_tear_kernel<double><<<ceil_div(n, 256), 256, 0, s>>>(n, d, e);
  count_launch(2);
  cudaMemsetAsync(W.Qalt, 0, sizeof(double) * (size_t)n * n, s);
  double *Qin = Q, *Qout = W.Qalt;
  for (int L = 1; L <= nlev; ++L) {
    const Merge *dm = reinterpret_cast<const Merge *>(meta + P.off_merge[L]);
    const int *pm = meta + P.off_pm[L];
    const int *pma = meta + P.off_pma[L];
    const int nm = P.nm[L];
    const int max_block = std::min(1 << L, n);
    dc_sort_kernel<double><<<nm, 256, 0, s>>>(dm, d, e, Qin, n, W);
    const int sn = dc_stage_n<double>(max_block);   // max_block <= 256: under the default 48 KB
    dc_deflate_kernel<double><<<nm, 256, dc_stage_bytes<double>(sn), s>>>(dm, e, W, sn);
    dc_group_kernel<double><<<nm, 256, 0, s>>>(dm, W);
    count_launch();
    dim3 gr(nm, ceil_div(max_block, 256));
    dc_rotate_kernel<double><<<gr, 256, 0, s>>>(dm, Qin, n, W);
    int wb = ceil_div((long long)n * 32, 256);
    dc_secular_kernel<double><<<wb, 256, 0, s>>>(n, dm, pm, e, W, status);
    dc_zhat_kernel<double><<<wb, 256, 0, s>>>(n, dm, pm, e, W);
    dc_build_u_kernel<double><<<wb, 256, 0, s>>>(n, dm, pm, W, n);
    dc_gather_kernel<double><<<n, 128, 0, s>>>(n, dm, pm, Qin, n, W, n);
    count_launch(7);
    if (max_block <= kSmallMerge) {
      dc_small_gemm_kernel<double><<<nm, 256, 0, s>>>(dm, W, n);
      count_launch();
    } else {
      // at most two merges at this size (n <= 256): read their sizes into a stack buffer
      int hK[2] = {0, 0};
      cudaMemcpyAsync(hK, W.mK, sizeof(int) * std::min(nm, 2), cudaMemcpyDeviceToHost, s);
      cudaStreamSynchronize(s);
      for (int k = 0; k < std::min(nm, 2); ++k) {
        int a = k << L, b = std::min(a + (1 << L), n), m = std::min(a + (1 << (L - 1)), b);
        if (m == b || hK[k] == 0) continue;
        dgemm(s, 'N', 'N', b - a, hK[k], hK[k], 1.0, W.Gs + a + (size_t)a * n, n, W.U + (size_t)a * n, n, 0.0,
              W.Qtmp + a + (size_t)a * n, n);
      }
    }
    dim3 grk(nm, ceil_div(max_block, 256));
    dc_rank_kernel<double><<<grk, 256, 0, s>>>(dm, d, W);
    dc_scatter_kernel<double><<<n, 128, 0, s>>>(n, pma, dm, Qin, n, Qout, d, W, n);
    count_launch(2);
    std::swap(Qin, Qout);
  }
  if (Qin != Q) cudaMemcpyAsync(Q, Qin, sizeof(double) * (size_t)n * n, cudaMemcpyDeviceToDevice, s);
  int st = 0;
  cudaMemcpyAsync(&st, status, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  return st;
}

}  // namespace dg

// Per-device address of the scratch array, resolved once per device on the first call.
static double *g_noalloc_dev_ptr[64] = {nullptr};

extern "C" int dftbgpu_stedc_noalloc(int n, double *d, const double *e, double *q, void *stream) {
  if (n < 1 || n > dg::kNoAllocMaxN || !d || !q || (n > 1 && !e)) return DFTBGPU_ERR_ARGS;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return DFTBGPU_ERR_CUDA;
  if (!g_noalloc_dev_ptr[dev]) {
    double *ptr = nullptr;
    if (cudaGetSymbolAddress((void **)&ptr, dg::g_noalloc_scratch) != cudaSuccess || !ptr) return DFTBGPU_ERR_CUDA;
    g_noalloc_dev_ptr[dev] = ptr;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the merge products go through dgemm; with the calling thread's tensor-core routing flag set it
  // would send them to tc_dgemm, whose per-thread scratch is allocated on first use. Keep the FP64
  // FMA kernel (no workspace) for this call.
  const bool tc_route = dg::g_tc_dgemm;
  dg::g_tc_dgemm = false;
  int st = dg::stedc_noalloc_impl(s, n, d, e, q, g_noalloc_dev_ptr[dev]);
  dg::g_tc_dgemm = tc_route;
  if (cudaGetLastError() != cudaSuccess) return DFTBGPU_ERR_CUDA;
  if (st == dg::kDevIterCap) return DFTBGPU_ERR_ITER_CAP;
  return st == 0 ? DFTBGPU_OK : DFTBGPU_ERR_CUDA;
}
