// Batched SCC-DFTB kernels (one CTA per molecule) and their host drivers.
#include <algorithm>
#include <cfloat>
#include <cstring>
#include <numeric>

#include "batch.cuh"
#include "dftb_device.cuh"

namespace dg {

// ------------------------------------------------------------------------------ CTA helpers
template <typename T>
__device__ __forceinline__ T wsum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum (fixed order; every thread gets the result). sh: 33 elements.
template <typename T>
__device__ T cta_sum(T v, T *sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = wsum(v);
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    T r = (lane < nw) ? sh[lane] : T(0);
    r = wsum(r);
    if (lane == 0) sh[32] = r;
  }
  __syncthreads();
  return sh[32];
}

__device__ double cta_max(double v, double *sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double r = (lane < nw) ? sh[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r = fmax(r, __shfl_xor_sync(0xffffffffu, r, o));
    if (lane == 0) sh[32] = r;
  }
  __syncthreads();
  return sh[32];
}

// Block-wide compensated (Neumaier) sum; sh_s, sh_c: 33 elements each.
__device__ double cta_csum(Comp v, double *sh_s, double *sh_c) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    double os = __shfl_xor_sync(0xffffffffu, v.s, o);
    double oc = __shfl_xor_sync(0xffffffffu, v.c, o);
    neumaier(v, os);
    v.c += oc;
  }
  __syncthreads();
  if (lane == 0) {
    sh_s[w] = v.s;
    sh_c[w] = v.c;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    Comp u = {lane < nw ? sh_s[lane] : 0.0, lane < nw ? sh_c[lane] : 0.0};
    for (int o = 16; o > 0; o >>= 1) {
      double os = __shfl_xor_sync(0xffffffffu, u.s, o);
      double oc = __shfl_xor_sync(0xffffffffu, u.c, o);
      neumaier(u, os);
      u.c += oc;
    }
    if (lane == 0) sh_s[32] = u.s + u.c;
  }
  __syncthreads();
  return sh_s[32];
}

struct MolV {
  int id, nat, n, a0, o0;
  long long mo, go;
};
__device__ __forceinline__ MolV mol_view(const BatchDev &B, int id) {
  MolV v;
  v.id = id;
  v.a0 = B.atom_off[id];
  v.nat = B.atom_off[id + 1] - v.a0;
  v.o0 = B.orb_off[id];
  v.n = B.orb_off[id + 1] - v.o0;
  v.mo = B.mat_off[id];
  v.go = B.gam_off[id];
  return v;
}

// Tiled product C = alpha op(A) op(B) + beta C computed by one CTA of 256 threads (32 x 32 tiles of
// C, 4 outputs per thread, K in steps of 32 through shared memory). Triangular flags only skip
// tiles and K blocks that are structurally zero; the skipped operand parts must hold zeros.
enum : int { kGLowerC = 1, kGALower = 2, kGAUpper = 4, kGBLower = 8 };
constexpr int GT = 32;

template <typename TI, typename TO>
__device__ void cta_gemm(int m, int n, int k, TI alpha, const TI *A, int lda, bool ta, const TI *B, int ldb,
                         bool tb, TI beta, TO *C, int ldc, int flags, TI (*As)[GT + 1], TI (*Bs)[GT + 1]) {
  const int t = threadIdx.x;
  const int r = t & 31, cg = t >> 5;
  const int mt = (m + GT - 1) / GT, nt = (n + GT - 1) / GT;
  for (int tile = 0; tile < mt * nt; ++tile) {
    const int i0 = (tile % mt) * GT, j0 = (tile / mt) * GT;
    if ((flags & kGLowerC) && j0 > i0 + GT - 1) continue;
    int kmin = 0, kmax = k;
    if (flags & kGALower) kmax = min(kmax, i0 + GT);
    if (flags & kGAUpper) kmin = max(kmin, i0);
    if (flags & kGBLower) kmin = max(kmin, j0);
    kmin = (kmin / GT) * GT;
    TI acc[4] = {TI(0), TI(0), TI(0), TI(0)};
    for (int k0 = kmin; k0 < kmax; k0 += GT) {
      __syncthreads();
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int e = t + 256 * q;
        {
          const int rr = ta ? (e >> 5) : (e & 31), cc = ta ? (e & 31) : (e >> 5);
          const int gi = i0 + rr, gk = k0 + cc;
          TI v = TI(0);
          if (gi < m && gk < k) v = ta ? A[gk + (size_t)gi * lda] : A[gi + (size_t)gk * lda];
          As[rr][cc] = v;
        }
        {
          const int rr = tb ? (e >> 5) : (e & 31), cc = tb ? (e & 31) : (e >> 5);
          const int gk = k0 + rr, gj = j0 + cc;
          TI v = TI(0);
          if (gk < k && gj < n) v = tb ? B[gj + (size_t)gk * ldb] : B[gk + (size_t)gj * ldb];
          Bs[rr][cc] = v;
        }
      }
      __syncthreads();
#pragma unroll 8
      for (int kk = 0; kk < GT; ++kk) {
        const TI a = As[r][kk];
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q] = fma(a, Bs[kk][cg * 4 + q], acc[q]);
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = i0 + r, j = j0 + cg * 4 + q;
      if (i < m && j < n && (!(flags & kGLowerC) || i >= j)) {
        TI v = alpha * acc[q];
        if (beta != TI(0)) v += beta * (TI)C[i + (size_t)j * ldc];
        C[i + (size_t)j * ldc] = (TO)v;
      }
    }
  }
  __syncthreads();
}

// ------------------------------------------------------------------------------ geometry
// Per molecule (one CTA): H0/S blocks (nonscc.F90:66-181 over all pairs within the molecule inside
// the SK cutoff), gamma matrix (coulomb.F90:704-733 1/r and shortgamma.F90:804-858 short part, U on
// the diagonal), repulsive energy, reference charges, Cholesky factor L of S, L^-1 and
// A0 = L^-1 H0 L^-T, plus FP32 copies of L, L^-1 and A0 for the mixed form.
__global__ void __launch_bounds__(kBatchThreads) batch_geom_kernel(ModelDev M, BatchDev B, double cut2) {
  __shared__ WarpSk ws_all[kBatchThreads / 32];
  __shared__ double sh[33], sh2[33];
  __shared__ double As[GT][GT + 1], Bs[GT][GT + 1];
  __shared__ int s_fail;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31, bd = blockDim.x, nwarp = bd >> 5;
  const MolV mv = mol_view(B, B.order[blockIdx.x]);
  const int n = mv.n, nat = mv.nat;
  MolState &st = B.st[mv.id];
  double *H0 = B.H0 + mv.mo, *S = B.S + mv.mo, *L = B.L + mv.mo, *Li = B.Li + mv.mo, *A0 = B.A0 + mv.mo;
  double *T = B.T + mv.mo;
  const size_t nn = (size_t)n * n;
  for (size_t i = t; i < nn; i += bd) {
    H0[i] = 0.0;
    S[i] = 0.0;
  }
  __syncthreads();
  for (int a = t; a < nat; a += bd) {
    const int ga = mv.a0 + a;
    const SpeciesDev &sp = M.sp[B.species[ga]];
    const int o = B.a_orb[ga] - mv.o0;
    int kq = 0;
    double q0 = 0.0;
    for (int s = 0; s < sp.n_shell; ++s) {
      q0 += sp.occ[s];
      for (int q = 0; q < 2 * sp.ang[s] + 1; ++q, ++kq) {
        H0[(size_t)(o + kq) * (n + 1)] = sp.onsite[s];
        S[(size_t)(o + kq) * (n + 1)] = 1.0;
      }
    }
    B.q0[ga] = q0;
  }
  for (int i = 0; i < nat; ++i) {
    for (int j = i + 1 + warp; j < nat; j += nwarp) {
      const int gi = mv.a0 + i, gj = mv.a0 + j;
      const double vx = B.xyz[3 * gj] - B.xyz[3 * gi];
      const double vy = B.xyz[3 * gj + 1] - B.xyz[3 * gi + 1];
      const double vz = B.xyz[3 * gj + 2] - B.xyz[3 * gi + 2];
      if (vx * vx + vy * vy + vz * vz > cut2) continue;
      const int si = B.species[gi], sj = B.species[gj];
      WarpSk &ws = ws_all[warp];
      eval_blocks(M, si, sj, vx, vy, vz, ws, lane);
      const int oi = B.a_orb[gi] - mv.o0, oj = B.a_orb[gj] - mv.o0;
      const int ni = M.sp[si].n_orb, nj = M.sp[sj].n_orb;
      for (int idx = lane; idx < ni * nj; idx += 32) {
        const int b = idx % nj, a = idx / nj;
        const double hv = ws.blk[0][b][a], sv = ws.blk[1][b][a];
        H0[(oj + b) + (size_t)(oi + a) * n] = hv;
        H0[(oi + a) + (size_t)(oj + b) * n] = hv;
        S[(oj + b) + (size_t)(oi + a) * n] = sv;
        S[(oi + a) + (size_t)(oj + b) * n] = sv;
      }
      __syncwarp();
    }
  }
  // gamma (column b contiguous in a) and repulsive energy per atom
  double *gam = B.gam + mv.go;
  for (int idx = t; idx < nat * nat; idx += bd) {
    const int a = idx % nat, b = idx / nat;
    const int ga = mv.a0 + a, gb = mv.a0 + b;
    const int sa = B.species[ga], sb = B.species[gb];
    const double ua = M.sp[sa].hubbu;
    double g;
    if (a == b) {
      g = -exp_gamma(0.0, ua, ua);
    } else {
      const double dx = B.xyz[3 * ga] - B.xyz[3 * gb], dy = B.xyz[3 * ga + 1] - B.xyz[3 * gb + 1],
                   dz = B.xyz[3 * ga + 2] - B.xyz[3 * gb + 2];
      const double r2 = dx * dx + dy * dy + dz * dz, r = sqrt(r2);
      g = 1.0 / r;
      const double rc = M.pair[sa * M.nsp + sb].gamma_cut;
      if (r2 <= rc * rc + kTolSameDist * kTolSameDist) g -= exp_gamma(r, M.sp[sb].hubbu, ua);
    }
    gam[a + (size_t)b * nat] = g;
  }
  Comp ce = {0.0, 0.0};
  for (int a = t; a < nat; a += bd) {
    const int ga = mv.a0 + a;
    const int sa = B.species[ga];
    double s = 0.0;
    for (int b = 0; b < nat; ++b) {
      if (b == a) continue;
      const int gb = mv.a0 + b;
      const double dx = B.xyz[3 * ga] - B.xyz[3 * gb], dy = B.xyz[3 * ga + 1] - B.xyz[3 * gb + 1],
                   dz = B.xyz[3 * ga + 2] - B.xyz[3 * gb + 2];
      const PairDev &P = M.pair[B.species[gb] * M.nsp + sa];
      const double r2 = dx * dx + dy * dy + dz * dz;
      if (r2 > P.rep_cut * P.rep_cut) continue;
      double e, de;
      spline_rep(M.rep + P.off_rep, P.n_spline, sqrt(r2), &e, &de);
      s += 0.5 * e;
    }
    B.erep[ga] = s;
    neumaier(ce, s);
  }
  const double erep = cta_csum(ce, sh, sh2);
  __syncthreads();
  // Cholesky S = L L^T (right-looking, lower)
  for (size_t i = t; i < nn; i += bd) L[i] = S[i];
  if (t == 0) s_fail = 0;
  for (int j = 0; j < n; ++j) {
    __syncthreads();
    if (t == 0) {
      double dj = L[j + (size_t)j * n];
      if (!(dj > 0.0)) {
        s_fail = 1;
        dj = 1.0;
      }
      dj = sqrt(dj);
      L[j + (size_t)j * n] = dj;
      sh[0] = 1.0 / dj;
    }
    __syncthreads();
    const double inv = sh[0];
    for (int i = j + 1 + t; i < n; i += bd) L[i + (size_t)j * n] *= inv;
    __syncthreads();
    const int m = n - j - 1;
    for (int idx = t; idx < m * m; idx += bd) {
      const int ii = j + 1 + idx % m, jj = j + 1 + idx / m;
      if (ii >= jj) L[ii + (size_t)jj * n] -= L[ii + (size_t)j * n] * L[jj + (size_t)j * n];
    }
  }
  __syncthreads();
  for (size_t idx = t; idx < nn; idx += bd) {
    const int i = (int)(idx % n), j = (int)(idx / n);
    if (i < j) L[idx] = 0.0;
    T[j + (size_t)i * n] = (i >= j) ? L[idx] : 0.0;   // T = L^T: row i of L contiguous
  }
  __syncthreads();
  // L^-1 by forward substitution, one column per thread
  for (int c = t; c < n; c += bd) {
    double *x = Li + (size_t)c * n;
    for (int i = 0; i < c; ++i) x[i] = 0.0;
    for (int i = c; i < n; ++i) {
      const double *lrow = T + (size_t)i * n;
      double s = (i == c) ? 1.0 : 0.0;
      for (int kk = c; kk < i; ++kk) s -= lrow[kk] * x[kk];
      x[i] = s / lrow[i];
    }
  }
  __syncthreads();
  // A0 = L^-1 (H0 L^-T): lower triangle, then mirrored
  cta_gemm<double, double>(n, n, n, 1.0, H0, n, false, Li, n, true, 0.0, T, n, 0, As, Bs);
  cta_gemm<double, double>(n, n, n, 1.0, Li, n, false, T, n, false, 0.0, A0, n, kGLowerC | kGALower, As, Bs);
  for (size_t idx = t; idx < nn; idx += bd) {
    const int i = (int)(idx % n), j = (int)(idx / n);
    if (i < j) A0[idx] = A0[j + (size_t)i * n];
  }
  __syncthreads();
  float *L32 = B.L32 + mv.mo, *Li32 = B.Li32 + mv.mo, *A032 = B.A0_32 + mv.mo;
  for (size_t idx = t; idx < nn; idx += bd) {
    L32[idx] = (float)L[idx];
    Li32[idx] = (float)Li[idx];
    A032[idx] = (float)A0[idx];
  }
  if (t == 0) {
    st.erep = erep;
    st.status = s_fail ? (int)kDevNotPosDef : 0;
    st.n_iter = 0;
    st.conv = 0;
  }
}

// ------------------------------------------------------------------------------ eigensolver
template <typename T>
struct Lim;
template <>
struct Lim<double> {
  static __device__ __forceinline__ double eps() { return DBL_EPSILON; }
};
template <>
struct Lim<float> {
  static __device__ __forceinline__ float eps() { return FLT_EPSILON; }
};

// Householder reduction of the full symmetric A (n x n, destroyed) to tridiagonal form
// (d[n], e[n-1]) with the reflector vectors kept in the columns of A below the subdiagonal
// (LAPACK dsytd2 semantics, lower: H = I - tau v v^T, v(0) = 1, beta = -sign(alpha) ||x||), followed
// by the explicit accumulation Q = H_0 ... H_{n-3} into Q (n x n). sv, sw: shared vectors of n.
template <typename T>
__device__ void cta_tridiag(int n, T *A, T *Q, T *d, T *e, T *sv, T *sw, T *sh) {
  const int t = threadIdx.x, bd = blockDim.x, lane = t & 31, warp = t >> 5, nw = bd >> 5;
  __shared__ T s_par[4];
  for (int j = 0; j + 2 < n; ++j) {
    const int m = n - j - 1;
    T *colj = A + (size_t)j * n;
    T sig = T(0);
    for (int i = j + 2 + t; i < n; i += bd) sig = fma(colj[i], colj[i], sig);
    sig = cta_sum(sig, sh);
    if (t == 0) {
      const T alpha = colj[j + 1];
      T beta, tau, scale;
      if (sig == T(0)) {
        tau = T(0);
        beta = alpha;
        scale = T(0);
      } else {
        beta = -copysign(sqrt(alpha * alpha + sig), alpha);
        tau = (beta - alpha) / beta;
        scale = T(1) / (alpha - beta);
      }
      d[j] = colj[j];
      e[j] = beta;
      s_par[0] = tau;
      s_par[1] = scale;
    }
    __syncthreads();
    const T tau = s_par[0], scale = s_par[1];
    for (int i = t; i < m; i += bd) {
      const T v = (i == 0) ? T(1) : colj[j + 1 + i] * scale;
      sv[i] = v;
      if (i > 0) colj[j + 1 + i] = v;
    }
    __syncthreads();
    if (t == 0) colj[j + 1] = tau;   // tau of reflector j kept on the subdiagonal slot of column j
    if (tau != T(0)) {
      // p = tau A22 v (column i of A22 contiguous; one warp per column)
      T *A22 = A + (j + 1) + (size_t)(j + 1) * n;
      for (int i = warp; i < m; i += nw) {
        const T *ci = A22 + (size_t)i * n;
        T s = T(0);
        for (int k = lane; k < m; k += 32) s = fma(ci[k], sv[k], s);
        s = wsum(s);
        if (lane == 0) sw[i] = tau * s;
      }
      __syncthreads();
      T pv = T(0);
      for (int i = t; i < m; i += bd) pv = fma(sw[i], sv[i], pv);
      pv = cta_sum(pv, sh);
      const T K = T(-0.5) * tau * pv;
      for (int i = t; i < m; i += bd) sw[i] = fma(K, sv[i], sw[i]);
      __syncthreads();
      for (int idx = t; idx < m * m; idx += bd) {
        const int ii = idx % m, jj = idx / m;
        A22[ii + (size_t)jj * n] -= sv[ii] * sw[jj] + sw[ii] * sv[jj];
      }
    }
    __syncthreads();
  }
  if (t == 0) {
    if (n >= 2) {
      d[n - 2] = A[(n - 2) + (size_t)(n - 2) * n];
      e[n - 2] = A[(n - 1) + (size_t)(n - 2) * n];
    }
    d[n - 1] = A[(n - 1) + (size_t)(n - 1) * n];
  }
  // Q = H_0 (H_1 (... H_{n-3})) applied to the identity from the innermost reflector outwards
  for (size_t idx = t; idx < (size_t)n * n; idx += bd) Q[idx] = ((idx % n) == (idx / n)) ? T(1) : T(0);
  __syncthreads();
  for (int j = n - 3; j >= 0; --j) {
    const int m = n - j - 1;
    const T *colj = A + (size_t)j * n;
    const T tau = colj[j + 1];
    if (tau == T(0)) continue;
    for (int i = t; i < m; i += bd) sv[i] = (i == 0) ? T(1) : colj[j + 1 + i];
    __syncthreads();
    T *Q22 = Q + (j + 1) + (size_t)(j + 1) * n;
    for (int c = warp; c < m; c += nw) {
      const T *qc = Q22 + (size_t)c * n;
      T s = T(0);
      for (int k = lane; k < m; k += 32) s = fma(qc[k], sv[k], s);
      s = wsum(s);
      if (lane == 0) sw[c] = tau * s;
    }
    __syncthreads();
    for (int idx = t; idx < m * m; idx += bd) {
      const int ii = idx % m, jj = idx / m;
      Q22[ii + (size_t)jj * n] -= sv[ii] * sw[jj];
    }
    __syncthreads();
  }
}

// Implicit QL with shifts on the symmetric tridiagonal (d, e), eigenvectors accumulated into the
// columns of Z (n x n): for each eigenvalue in turn, sweeps with the shift from the leading 2 x 2
// until the coupling e(l) is negligible. Thread 0 generates the Givens rotations of a sweep (a short
// scalar recurrence), then every thread applies them to its rows of Z. Returns 0, or kDevIterCap if
// an eigenvalue needs more than kQlMaxIter sweeps. rc, rs: shared vectors of n.
constexpr int kQlMaxIter = 60;
template <typename T>
__device__ int cta_tql(int n, T *d, T *e, T *Z, T *rc, T *rs) {
  __shared__ int s_lo, s_hi, s_state;
  const int t = threadIdx.x, bd = blockDim.x;
  if (t == 0) {
    e[n - 1] = T(0);
    s_state = 0;
  }
  __syncthreads();
  for (int l = 0; l < n; ++l) {
    int iter = 0;
    while (true) {
      if (t == 0) {
        int m = l;
        for (; m < n - 1; ++m) {
          const T dd = fabs(d[m]) + fabs(d[m + 1]);
          if (fabs(e[m]) <= Lim<T>::eps() * dd) break;
        }
        if (m == l) {
          s_lo = -1;   // converged
        } else if (++iter > kQlMaxIter) {
          s_lo = -1;
          s_state = (int)kDevIterCap;
        } else {
          T g = (d[l + 1] - d[l]) / (T(2) * e[l]);
          T r = hypot(g, T(1));
          g = d[m] - d[l] + e[l] / (g + copysign(r, g));
          T s = T(1), c = T(1), p = T(0);
          int i = m - 1;
          bool broke = false;
          for (; i >= l; --i) {
            const T f = s * e[i], b = c * e[i];
            r = sqrt(fma(f, f, g * g));   // entries are O(1): no scaling needed
            e[i + 1] = r;
            if (r == T(0)) {
              d[i + 1] -= p;
              e[m] = T(0);
              broke = true;
              break;
            }
            const T ir = T(1) / r;
            s = f * ir;
            c = g * ir;
            g = d[i + 1] - p;
            r = (d[i] - g) * s + T(2) * c * b;
            p = s * r;
            d[i + 1] = g + p;
            g = c * r - b;
            rc[i] = c;
            rs[i] = s;
          }
          if (!broke) {
            d[l] -= p;
            e[l] = g;
            e[m] = T(0);
          }
          s_lo = broke ? i + 1 : l;   // rotations rc/rs[s_lo .. m-1] were generated
          s_hi = m - 1;
        }
      }
      __syncthreads();
      const int lo = s_lo, hi = s_hi;
      if (lo < 0) break;
      if (lo <= hi) {
        // rows are independent: each thread streams its rows through the rotations, four column
        // loads in flight ahead of the dependent rotation chain
        for (int k = t; k < n; k += bd) {
          T *zr = Z + k;
          T carry = zr[(size_t)(hi + 1) * n];
          int i = hi;
          for (; i - 3 >= lo; i -= 4) {
            const T z0 = zr[(size_t)i * n], z1 = zr[(size_t)(i - 1) * n];
            const T z2 = zr[(size_t)(i - 2) * n], z3 = zr[(size_t)(i - 3) * n];
            zr[(size_t)(i + 1) * n] = fma(rs[i], z0, rc[i] * carry);
            carry = fma(rc[i], z0, -rs[i] * carry);
            zr[(size_t)i * n] = fma(rs[i - 1], z1, rc[i - 1] * carry);
            carry = fma(rc[i - 1], z1, -rs[i - 1] * carry);
            zr[(size_t)(i - 1) * n] = fma(rs[i - 2], z2, rc[i - 2] * carry);
            carry = fma(rc[i - 2], z2, -rs[i - 2] * carry);
            zr[(size_t)(i - 2) * n] = fma(rs[i - 3], z3, rc[i - 3] * carry);
            carry = fma(rc[i - 3], z3, -rs[i - 3] * carry);
          }
          for (; i >= lo; --i) {
            const T zi = zr[(size_t)i * n];
            zr[(size_t)(i + 1) * n] = fma(rs[i], zi, rc[i] * carry);
            carry = fma(rc[i], zi, -rs[i] * carry);
          }
          zr[(size_t)lo * n] = carry;
        }
      }
      __syncthreads();
    }
    __syncthreads();
  }
  return s_state;
}

// Ascending order: eig[rank(i)] = d[i] (double), Y[:, rank(i)] = Z[:, i]. perm: shared ints of n.
template <typename T>
__device__ void cta_sort_eig(int n, const T *d, const T *Z, double *eig, T *Y, int *perm) {
  const int t = threadIdx.x, bd = blockDim.x;
  for (int i = t; i < n; i += bd) {
    const T di = d[i];
    int r = 0;
    for (int j = 0; j < n; ++j) {
      const T dj = d[j];
      r += (dj < di || (dj == di && j < i)) ? 1 : 0;
    }
    perm[r] = i;
    eig[r] = (double)di;
  }
  __syncthreads();
  for (size_t idx = t; idx < (size_t)n * n; idx += bd) {
    const int rr = (int)(idx % n), c = (int)(idx / n);
    Y[idx] = Z[rr + (size_t)perm[c] * n];
  }
  __syncthreads();
}

// ------------------------------------------------------------------------------ Fermi filling
// etemp.F90:59-191 for one molecule (same steps as the single-system kernel: mid-gap try for integer
// electron counts, bracketing, bisection to elecTol, compensated sums, rescaling), on one CTA.
__device__ double cta_electron_count(int n, const double *eig, double ef, double beta, double *sh_s,
                                     double *sh_c) {
  Comp c = {0.0, 0.0};
  for (int j = threadIdx.x; j < n; j += blockDim.x) neumaier(c, 1.0 / (1.0 + exp((eig[j] - ef) * beta)));
  return cta_csum(c, sh_s, sh_c);
}

__device__ int cta_fermi(int n, const double *eig, double nel_total, double kT, double *fill, MolState &st,
                         double *sh_s, double *sh_c, int *sh_i) {
  const double nel = 0.5 * nel_total;
  const double beta = 1.0 / kT;
  const double eps2 = 2.0 * kEps;
  double ef;
  int status = 0;
  bool rescale = false;
  double ne_final = nel;
  if ((double)n <= nel) {
    ef = eig[n - 1] + 1000.0 * (kT + (double)FLT_EPSILON);
  } else {
    bool done = false;
    if (fabs(nel - rint(nel)) <= kElecTol) {
      int nocc = (int)ceil(nel - 1e-12);
      if (nocc < 1) nocc = 1;
      const int lumo = min(n, nocc + 1) - 1;
      ef = 0.5 * (eig[lumo] + eig[nocc - 1]);
      const double ne = cta_electron_count(n, eig, ef, beta, sh_s, sh_c);
      if (fabs(nel - ne) <= kElecTolMax) done = true;
    }
    if (!done) {
      double up = eig[n - 1] + 0.01, lo = eig[0] - 0.01;
      double nmax = cta_electron_count(n, eig, up, beta, sh_s, sh_c);
      double nmin = cta_electron_count(n, eig, lo, beta, sh_s, sh_c);
      int guard = 0;
      while (nmin > nel && guard++ < 200) {
        lo = 2.0 * (lo - up) + lo;
        nmin = cta_electron_count(n, eig, lo, beta, sh_s, sh_c);
      }
      while (nmax < nel && guard++ < 400) {
        up = 2.0 * (up - lo) + lo;
        nmax = cta_electron_count(n, eig, up, beta, sh_s, sh_c);
      }
      ef = 0.5 * (up + lo);
      double ne = cta_electron_count(n, eig, ef, beta, sh_s, sh_c);
      int it = 0;
      while (fabs(nel - ne) > kElecTol && fabs(up - lo) >= fmax(fabs(ef) * eps2, eps2) && it++ < 2000) {
        if ((nmax >= nmin) == (nel >= ne)) {
          lo = ef;
          nmin = ne;
        } else {
          up = ef;
          nmax = ne;
        }
        ef = 0.5 * (up + lo);
        ne = cta_electron_count(n, eig, ef, beta, sh_s, sh_c);
      }
      if (fabs(nel - ne) > kElecTolMax) status = kDevFermiFail;
      ne = cta_electron_count(n, eig, ef, beta, sh_s, sh_c);
      if (nel > eps2 && fabs(nel - ne) > eps2) {
        rescale = true;
        ne_final = ne;
      }
    }
  }
  if (threadIdx.x == 0) *sh_i = n;
  __syncthreads();
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const double f = 1.0 / (1.0 + exp((eig[j] - ef) * beta));
    if (f <= kElecTol) atomicMin(sh_i, j);
  }
  __syncthreads();
  const int j0 = *sh_i;
  Comp cb = {0.0, 0.0}, ct = {0.0, 0.0};
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    double f = 0.0;
    if (j <= j0) {
      f = 1.0 / (1.0 + exp((eig[j] - ef) * beta));
      if (f > kEps && f < 1.0 - kEps) neumaier(ct, -(f * log(f) + (1.0 - f) * log(1.0 - f)));
      neumaier(cb, f * eig[j]);
    }
    if (rescale) f = f * nel / ne_final;
    fill[j] = 2.0 * f;
  }
  const double eb = cta_csum(cb, sh_s, sh_c);
  const double ts = cta_csum(ct, sh_s, sh_c) * kT;
  __syncthreads();
  if (threadIdx.x == 0) *sh_i = 0;
  __syncthreads();
  for (int j = threadIdx.x; j < n; j += blockDim.x)
    if (fabs(fill[j]) >= kEps) atomicMax(sh_i, j + 1);
  __syncthreads();
  const int k = *sh_i;
  if (threadIdx.x == 0) {
    st.ef = ef;
    st.eband = 2.0 * eb;
    st.ts = 2.0 * ts;
    st.e0 = 2.0 * (eb - 0.5 * ts);
    st.k = k;
  }
  __syncthreads();
  return status;
}

// ------------------------------------------------------------------------------ Broyden
// mixer/broydenmixer.F90:204-342 (modified Broyden) for one molecule on one CTA, the same steps as
// the single-system mixer; the convergence test max|q_out - q_in| < tol (main.F90:4907-4908) decides
// whether a mixing step is taken. History (ww, aa, dF, uu) and the small linear system (beta, cc)
// live in the molecule's slices of global memory. Returns the SCC error; *conv receives the flag.
struct BroydenMol {
  double *ww, *aa, *beta, *cc, *dF, *uu, *qlast, *dlast;
  int M;
};

__device__ double cta_broyden(int N, int it, int mix_it, int min_iter, int max_iter, double tol, const BatchOpts &o,
                              BroydenMol B, double *qin, const double *qout, bool *conv_out, double *sh) {
  const int t = threadIdx.x, bd = blockDim.x;
  double mx = 0.0;
  for (int i = t; i < N; i += bd) mx = fmax(mx, fabs(qout[i] - qin[i]));
  const double err = cta_max(mx, sh);
  const bool conv = (err < tol) && (it >= min_iter);
  *conv_out = conv;
  if (conv || it == max_iter) return err;
  const int nn = mix_it;
  if (nn > B.M) return err;
  if (nn == 1) {
    for (int i = t; i < N; i += bd) {
      const double d = qout[i] - qin[i];
      B.qlast[i] = qin[i];
      B.dlast[i] = d;
      qin[i] = qin[i] + o.alpha * d;
    }
    __syncthreads();
    return err;
  }
  const int n1 = nn - 1, M = B.M;
  double ss = 0.0;
  for (int i = t; i < N; i += bd) {
    const double d = qout[i] - qin[i];
    ss = fma(d, d, ss);
  }
  const double wn = sqrt(cta_sum(ss, sh));
  double ww = (wn > o.wfac / o.maxw) ? o.wfac / wn : o.maxw;
  if (ww < o.minw) ww = o.minw;
  if (t == 0) B.ww[n1 - 1] = ww;
  double s2 = 0.0;
  for (int i = t; i < N; i += bd) {
    const double v = (qout[i] - qin[i]) - B.dlast[i];
    s2 = fma(v, v, s2);
  }
  const double nrm = fmax(sqrt(cta_sum(s2, sh)), kEps);
  const double inv = 1.0 / nrm;
  double *df = B.dF + (size_t)(n1 - 1) * N;
  for (int i = t; i < N; i += bd) df[i] = inv * ((qout[i] - qin[i]) - B.dlast[i]);
  __syncthreads();
  double *cc = B.cc, *beta = B.beta;
  for (int i = 0; i < n1 - 1; ++i) {
    const double *dfi = B.dF + (size_t)i * N;
    double a = 0.0, c = 0.0;
    for (int k = t; k < N; k += bd) {
      a = fma(dfi[k], df[k], a);
      c = fma(dfi[k], qout[k] - qin[k], c);
    }
    a = cta_sum(a, sh);
    c = cta_sum(c, sh);
    if (t == 0) {
      B.aa[i + (size_t)(n1 - 1) * M] = a;
      B.aa[(n1 - 1) + (size_t)i * M] = a;
      cc[i] = B.ww[i] * c;
    }
  }
  {
    double c = 0.0;
    for (int k = t; k < N; k += bd) c = fma(df[k], qout[k] - qin[k], c);
    c = cta_sum(c, sh);
    if (t == 0) {
      B.aa[(n1 - 1) + (size_t)(n1 - 1) * M] = 1.0;
      cc[n1 - 1] = ww * c;
    }
  }
  __syncthreads();
  for (int idx = t; idx < n1 * n1; idx += bd) {
    const int i = idx % n1, j = idx / n1;
    double v = B.ww[i] * B.ww[j] * B.aa[i + (size_t)j * M];
    if (i == j) v += o.omega0 * o.omega0;
    beta[i + j * n1] = v;
  }
  __syncthreads();
  // Gaussian elimination with partial pivoting on beta x = cc
  __shared__ int piv;
  for (int k = 0; k < n1; ++k) {
    if (t == 0) {
      int p = k;
      double best = fabs(beta[k + k * n1]);
      for (int i = k + 1; i < n1; ++i)
        if (fabs(beta[i + k * n1]) > best) {
          best = fabs(beta[i + k * n1]);
          p = i;
        }
      piv = p;
    }
    __syncthreads();
    const int p = piv;
    if (p != k) {
      for (int j = t; j < n1; j += bd) {
        const double tmp = beta[k + j * n1];
        beta[k + j * n1] = beta[p + j * n1];
        beta[p + j * n1] = tmp;
      }
      if (t == 0) {
        const double tmp = cc[k];
        cc[k] = cc[p];
        cc[p] = tmp;
      }
    }
    __syncthreads();
    const double dkk = beta[k + k * n1];
    for (int idx = t; idx < (n1 - k - 1) * (n1 - k); idx += bd) {
      const int i = k + 1 + idx % (n1 - k - 1);
      const int j = k + idx / (n1 - k - 1);
      const double lik = beta[i + k * n1] / dkk;
      if (j > k) beta[i + j * n1] -= lik * beta[k + j * n1];
    }
    __syncthreads();
    if (t == 0)
      for (int i = k + 1; i < n1; ++i) cc[i] -= beta[i + k * n1] / dkk * cc[k];
    __syncthreads();
  }
  if (t == 0) {
    for (int i = n1 - 1; i >= 0; --i) {
      double v = cc[i];
      for (int j = i + 1; j < n1; ++j) v -= beta[i + j * n1] * cc[j];
      cc[i] = v / beta[i + i * n1];
    }
  }
  __syncthreads();
  double *u = B.uu + (size_t)(n1 - 1) * N;
  for (int i = t; i < N; i += bd) {
    const double qi = qin[i];
    const double d = qout[i] - qi;
    const double ui = o.alpha * df[i] + inv * (qi - B.qlast[i]);
    double nq = qi + o.alpha * d;
    for (int k = 0; k < n1 - 1; ++k) nq -= B.ww[k] * cc[k] * B.uu[(size_t)k * N + i];
    nq -= ww * cc[n1 - 1] * ui;
    B.qlast[i] = qi;
    B.dlast[i] = d;
    u[i] = ui;
    qin[i] = nq;
  }
  __syncthreads();
  return err;
}

// ------------------------------------------------------------------------------ SCC iteration
__device__ __forceinline__ void mats(const BatchDev &B, long long mo, double **L, double **Li, double **A0,
                                     double **A, double **Tm, double **Z) {
  *L = B.L + mo; *Li = B.Li + mo; *A0 = B.A0 + mo; *A = B.A + mo; *Tm = B.T + mo; *Z = B.Z + mo;
}
__device__ __forceinline__ void mats(const BatchDev &B, long long mo, float **L, float **Li, float **A0, float **A,
                                     float **Tm, float **Z) {
  *L = B.L32 + mo; *Li = B.Li32 + mo; *A0 = B.A0_32 + mo; *A = B.A32 + mo; *Tm = B.T32 + mo; *Z = B.Z32 + mo;
}

__global__ void batch_scc_init_kernel(BatchDev B, BatchOpts o) {
  __shared__ double sh[33];
  const int id = blockIdx.x;
  const MolV mv = mol_view(B, id);
  double s = 0.0;
  for (int a = threadIdx.x; a < mv.nat; a += blockDim.x) {
    B.qin[mv.a0 + a] = B.q0[mv.a0 + a];
    s += B.q0[mv.a0 + a];
  }
  s = cta_sum(s, sh);
  if (threadIdx.x == 0) {
    MolState &st = B.st[id];
    st.nel = s - o.net_charge;
    st.n_iter = 0;
    st.conv = 0;
    st.mix_calls = 0;
    st.form = o.mixed ? 1 : 0;
    st.err = 0.0;
    st.k = 0;
    st.verify = 0;
    st.pert_run = 0;
  }
}

// Common end of an SCC iteration of one molecule: Mulliken populations and Tr(rho H0)
// (populations.F90:120-191, getenergies.F90:198-199), output potentials, E_SCC and the molecule's
// Broyden step; thread 0 records the iteration in st. Returns the convergence flag (all threads).
__device__ bool cta_iter_tail(const BatchDev &B, const BatchOpts &o, const MolV &mv, int id, int it,
                              const double *rho, double *sh_s, double *sh_c) {
  const int t = threadIdx.x, bd = blockDim.x, lane = t & 31, warp = t >> 5, nw = bd >> 5;
  const int n = mv.n, nat = mv.nat;
  MolState &st = B.st[id];
  double *qin = B.qin + mv.a0, *qout = B.qout + mv.a0, *Vout = B.Vout + mv.a0;
  const double *q0 = B.q0 + mv.a0, *gam = B.gam + mv.go;
  // Mulliken (populations.F90:120-191) and Tr(rho H0) (getenergies.F90:198-199)
  double *qo = B.dd + mv.o0, *eo = B.ee + mv.o0;
  const double *S = B.S + mv.mo, *H0 = B.H0 + mv.mo;
  for (int mu = warp; mu < n; mu += nw) {
    const double *rc = rho + (size_t)mu * n, *scol = S + (size_t)mu * n, *hcol = H0 + (size_t)mu * n;
    double q = 0.0, e = 0.0;
    for (int nu = lane; nu < n; nu += 32) {
      q = fma(rc[nu], scol[nu], q);
      e = fma(rc[nu], hcol[nu], e);
    }
    q = wsum(q);
    e = wsum(e);
    if (lane == 0) {
      qo[mu] = q;
      eo[mu] = e;
    }
  }
  __syncthreads();
  for (int a = t; a < nat; a += bd) {
    const int ob = B.a_orb[mv.a0 + a] - mv.o0;
    const int oe = (a + 1 < nat) ? B.a_orb[mv.a0 + a + 1] - mv.o0 : n;
    double s = 0.0;
    for (int oo = ob; oo < oe; ++oo) s += qo[oo];
    qout[a] = s;
  }
  Comp ce = {0.0, 0.0};
  for (int oo = t; oo < n; oo += bd) neumaier(ce, eo[oo]);
  const double enonscc = cta_csum(ce, sh_s, sh_c);
  for (int a = t; a < nat; a += bd) {
    double s = 0.0;
    for (int b = 0; b < nat; ++b) s = fma(gam[a + (size_t)b * nat], qout[b] - q0[b], s);
    Vout[a] = s;
  }
  __syncthreads();
  Comp cs = {0.0, 0.0};
  for (int a = t; a < nat; a += bd) neumaier(cs, Vout[a] * (qout[a] - q0[a]));
  const double escc = 0.5 * cta_csum(cs, sh_s, sh_c);
  const int Mh = B.M;
  BroydenMol bm = {B.ww + (size_t)id * Mh, B.aa + (size_t)id * Mh * Mh, B.beta + (size_t)id * Mh * Mh,
                   B.cc + (size_t)id * Mh, B.dF + (size_t)mv.a0 * Mh, B.uu + (size_t)mv.a0 * Mh,
                   B.qlast + mv.a0, B.dlast + mv.a0, Mh};
  bool conv = false;
  const double err = cta_broyden(nat, it, st.mix_calls + 1, o.min_iter, o.max_iter, o.tol, o, bm, qin, qout, &conv,
                                 sh_s);
  __shared__ int s_conv;
  if (t == 0) {
    st.n_iter = it;
    st.err = err;
    st.enonscc = enonscc;
    st.escc = escc;
    if (!conv && it != o.max_iter) st.mix_calls += 1;
    s_conv = conv ? 1 : 0;
  }
  __syncthreads();
  return s_conv != 0;
}

// One SCC iteration of every eligible molecule (one CTA each): V = gamma dq_in, reduced
// A = A0 + 1/2 (B + B^T) with B = L^-1 diag(V) L, eigen-decomposition (Householder + implicit QL in
// precision T), Fermi filling, C = L^-T Y, rho = C f C^T, Mulliken populations, E_nonSCC, E_SCC and
// the molecule's Broyden step. FP32 molecules (mixed form) move to FP64 once their SCC error drops
// below switch_tol (the converged iteration is always FP64); the last allowed iteration is FP64.
// Molecules still active afterwards are counted in *active.
template <typename T>
__global__ void __launch_bounds__(kBatchThreads) batch_iter_kernel(ModelDev M, BatchDev B, BatchOpts o, int *active) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ T As[GT][GT + 1], Bs[GT][GT + 1];
  __shared__ double sh_s[33], sh_c[33];
  __shared__ T shT[33];
  __shared__ int sh_i;
  const int t = threadIdx.x, bd = blockDim.x;
  const int id = B.order[blockIdx.x];
  MolState &st = B.st[id];
  const bool is32 = sizeof(T) == 4;
  const int nit = st.n_iter;
  bool elig = st.status == 0 && !st.conv && nit < o.max_iter;
  if (is32) elig = elig && st.form == 1 && nit + 1 < o.max_iter;
  else elig = elig && (st.form == 0 || nit + 1 == o.max_iter);
  if (!elig) return;
  const MolV mv = mol_view(B, id);
  const int n = mv.n, nat = mv.nat, it = nit + 1;
  T *L, *Li, *A0, *A, *Tm, *Z;
  mats(B, mv.mo, &L, &Li, &A0, &A, &Tm, &Z);
  double *qin = B.qin + mv.a0, *V = B.V + mv.a0;
  const double *q0 = B.q0 + mv.a0, *gam = B.gam + mv.go;
  T *sv = reinterpret_cast<T *>(dsm), *sw = sv + n, *sd = sw + n, *se = sd + n;
  int *perm = reinterpret_cast<int *>(se + n);
  const size_t nn = (size_t)n * n;
  // potentials of the input charges
  for (int a = t; a < nat; a += bd) {
    double s = 0.0;
    for (int b = 0; b < nat; ++b) s = fma(gam[a + (size_t)b * nat], qin[b] - q0[b], s);
    V[a] = s;
  }
  __syncthreads();
  for (size_t idx = t; idx < nn; idx += bd) {
    const int i = (int)(idx % n), j = (int)(idx / n);
    Tm[idx] = (i >= j) ? (T)V[B.o_atom[mv.o0 + i] - mv.a0] * L[idx] : T(0);
  }
  __syncthreads();
  cta_gemm<T, T>(n, n, n, T(1), Li, n, false, Tm, n, false, T(0), Z, n, kGLowerC | kGALower | kGBLower, As, Bs);
  for (size_t idx = t; idx < nn; idx += bd) {
    const int i = (int)(idx % n), j = (int)(idx / n);
    const T bij = Z[max(i, j) + (size_t)min(i, j) * n];
    A[idx] = A0[idx] + ((i == j) ? bij : T(0.5) * bij);
  }
  __syncthreads();
  cta_tridiag<T>(n, A, Z, sd, se, sv, sw, shT);
  const int qs = cta_tql<T>(n, sd, se, Z, sv, sw);
  double *eig = B.eig + mv.o0, *fill = B.fill + mv.o0;
  cta_sort_eig<T>(n, sd, Z, eig, Tm, perm);
  const int fs = cta_fermi(n, eig, st.nel, o.kT, fill, st, sh_s, sh_c, &sh_i);
  const int k = st.k;
  double *rho = B.rho + mv.mo;
  // an FP64 iteration of the mixed form that is not a check of a perturbative state becomes the
  // reference of the perturbative updates: it keeps all n vectors
  const bool reference = !is32 && o.mixed && !st.verify;
  const int kc = reference ? n : k;
  if (kc > 0 && kc != k)
    cta_gemm<T, T>(n, kc, n, T(1), Li, n, true, Tm, n, false, T(0), Z, n, kGAUpper, As, Bs);
  if (k > 0) {
    if (kc == k) cta_gemm<T, T>(n, k, n, T(1), Li, n, true, Tm, n, false, T(0), Z, n, kGAUpper, As, Bs);
    for (size_t idx = t; idx < (size_t)n * k; idx += bd) A[idx] = Z[idx] * (T)fill[idx / n];
    __syncthreads();
    cta_gemm<T, double>(n, n, k, T(1), A, n, false, Z, n, true, T(0), rho, n, kGLowerC, As, Bs);
    for (size_t idx = t; idx < nn; idx += bd) {
      const int i = (int)(idx % n), j = (int)(idx / n);
      if (i < j) rho[idx] = rho[j + (size_t)i * n];
    }
  } else {
    for (size_t idx = t; idx < nn; idx += bd) rho[idx] = 0.0;
  }
  __syncthreads();
  if constexpr (sizeof(T) == 8) {
    if (reference) {
      // X = S C = L Y (Y: the sorted eigenvectors in Tm), FP32 copies of C and X, rho_ref, V_ref
      cta_gemm<T, T>(n, n, n, T(1), L, n, false, Tm, n, false, T(0), A, n, kGALower, As, Bs);
      float *X32 = B.X32 + mv.mo, *C32 = B.C32 + mv.mo;
      double *rref = B.rho_ref + mv.mo;
      for (size_t idx = t; idx < nn; idx += bd) {
        X32[idx] = (float)A[idx];
        C32[idx] = (float)Z[idx];
        rref[idx] = rho[idx];
      }
      for (int a = t; a < nat; a += bd) B.Vref[mv.a0 + a] = V[a];
      __syncthreads();
    }
  }
  const bool conv = cta_iter_tail(B, o, mv, id, it, rho, sh_s, sh_c);
  if (t == 0) {
    const int status = qs ? qs : fs;
    if (status) st.status = status;
    bool c = conv;
    if (is32) {
      if (conv || st.err < o.switch_tol) {
        st.form = 0;   // re-evaluated in FP64, never accepted in FP32
        c = false;
      }
    } else if (o.mixed && !c) {
      if (st.verify) {
        st.verify = 0;   // the check failed: the next FP64 iteration becomes a new reference
      } else if (reference) {
        st.form = 2;
        st.pert_run = 0;
      }
    }
    st.conv = c ? 1 : 0;
    if (!c && st.status == 0 && it < o.max_iter) atomicAdd(active, 1);
  }
}


// Perturbative SCC iteration of the mixed form for every molecule in that state (one CTA each):
// first-order density-matrix perturbation around the molecule's last FP64 reference (the same
// scheme as the single-system form): D = diag(V - V_ref), M = 1/2 (X^T D C + C^T D X) for the k
// occupied columns, dP_ij = K_ij (M_ij - dmu delta_ij) with the Fermi divided differences K,
// rho = rho_ref + C dP C^T, in FP32 per-CTA products (the operands carry the potential change only).
// A converged state is checked by an FP64 iteration with the occupied vectors; 16 perturbative
// iterations without convergence renew the reference.
constexpr int kBatchMaxPertRun = 16;
__global__ void __launch_bounds__(kBatchThreads) batch_pert_kernel(ModelDev M, BatchDev B, BatchOpts o, int *active) {
  __shared__ float As[GT][GT + 1], Bs[GT][GT + 1];
  __shared__ double sh_s[33], sh_c[33], s_dmu;
  const int t = threadIdx.x, bd = blockDim.x;
  const int id = B.order[blockIdx.x];
  MolState &st = B.st[id];
  const int nit = st.n_iter;
  if (!(st.status == 0 && !st.conv && st.form == 2 && nit + 1 < o.max_iter)) return;
  const MolV mv = mol_view(B, id);
  const int n = mv.n, nat = mv.nat, it = nit + 1, k = st.k;
  const size_t nn = (size_t)n * n;
  const double *qin = B.qin + mv.a0, *q0 = B.q0 + mv.a0, *gam = B.gam + mv.go, *Vref = B.Vref + mv.a0;
  double *V = B.V + mv.a0;
  const float *X = B.X32 + mv.mo, *Cf = B.C32 + mv.mo;
  float *DC = B.A32 + mv.mo, *DX = B.T32 + mv.mo, *Mt = B.Mt32 + mv.mo, *Zp = B.Zp32 + mv.mo, *D = B.Z32 + mv.mo;
  const double *eig = B.eig + mv.o0, *fill = B.fill + mv.o0, *rref = B.rho_ref + mv.mo;
  double *rho = B.rho + mv.mo;
  for (int a = t; a < nat; a += bd) {
    double s = 0.0;
    for (int b = 0; b < nat; ++b) s = fma(gam[a + (size_t)b * nat], qin[b] - q0[b], s);
    V[a] = s;
  }
  __syncthreads();
  for (size_t idx = t; idx < nn; idx += bd) {
    const int l = (int)(idx % n);
    const int a = B.o_atom[mv.o0 + l] - mv.a0;
    const float dv = (float)(V[a] - Vref[a]);
    DC[idx] = dv * Cf[idx];
    DX[idx] = dv * X[idx];
  }
  __syncthreads();
  if (k > 0) {
    cta_gemm<float, float>(n, k, n, 0.5f, DC, n, true, X, n, false, 0.f, Mt, n, 0, As, Bs);
    cta_gemm<float, float>(n, k, n, 0.5f, DX, n, true, Cf, n, false, 1.f, Mt, n, 0, As, Bs);
    // Fermi-level shift from charge conservation
    double num = 0.0, den = 0.0;
    for (int i = t; i < k; i += bd) {
      const double f = fill[i];
      const double fp = -f * (2.0 - f) / (2.0 * o.kT);
      num = fma(fp, (double)Mt[i + (size_t)i * n], num);
      den += fp;
    }
    num = cta_sum(num, sh_s);
    den = cta_sum(den, sh_c);
    if (t == 0) s_dmu = (fabs(den) > 1e-300) ? num / den : 0.0;
    __syncthreads();
    const double dmu = s_dmu;
    for (size_t idx = t; idx < (size_t)n * k; idx += bd) {
      const int j = (int)(idx % n), i = (int)(idx / n);
      const double fi = fill[i];
      double mij = (double)Mt[idx], K;
      if (j == i) {
        K = -fi * (2.0 - fi) / (2.0 * o.kT);
        mij -= dmu;
      } else {
        const double de = eig[i] - eig[j];
        if (fabs(de) > 1e-9) {
          K = (fi - fill[j]) / de;
        } else {
          const double fm = 0.5 * (fi + fill[j]);
          K = -fm * (2.0 - fm) / (2.0 * o.kT);
        }
      }
      double v = K * mij;
      if (j < k) v *= 0.5;
      Mt[idx] = (float)v;
    }
    __syncthreads();
    cta_gemm<float, float>(n, k, n, 1.f, Cf, n, false, Mt, n, false, 0.f, Zp, n, 0, As, Bs);
    cta_gemm<float, float>(n, n, k, 1.f, Zp, n, false, Cf, n, true, 0.f, D, n, kGLowerC, As, Bs);
    cta_gemm<float, float>(n, n, k, 1.f, Cf, n, false, Zp, n, true, 1.f, D, n, kGLowerC, As, Bs);
    for (size_t idx = t; idx < nn; idx += bd) {
      const int i = (int)(idx % n), j = (int)(idx / n);
      rho[idx] = rref[idx] + (double)((i >= j) ? D[idx] : D[j + (size_t)i * n]);
    }
  } else {
    for (size_t idx = t; idx < nn; idx += bd) rho[idx] = rref[idx];
  }
  __syncthreads();
  const bool conv = cta_iter_tail(B, o, mv, id, it, rho, sh_s, sh_c);
  if (t == 0) {
    if (conv) {
      st.form = 0;     // checked by an FP64 iteration at the same charges
      st.verify = 1;
    } else if (++st.pert_run >= kBatchMaxPertRun) {
      st.form = 0;     // renew the reference
    }
    st.conv = 0;
    if (st.status == 0 && it < o.max_iter) atomicAdd(active, 1);
  }
}

// ------------------------------------------------------------------------------ gradients
// Energy-weighted density matrix W = C diag(f eps) C^T per molecule (densitymatrix.F90:664-733),
// into the molecule's A buffer; C (n x k) is left in Z by the final (FP64) iteration.
__global__ void __launch_bounds__(kBatchThreads) batch_ew_kernel(BatchDev B) {
  __shared__ double As[GT][GT + 1], Bs[GT][GT + 1];
  const int id = B.order[blockIdx.x];
  const MolState &st = B.st[id];
  if (st.status != 0) return;
  const MolV mv = mol_view(B, id);
  const int n = mv.n, k = st.k, t = threadIdx.x, bd = blockDim.x;
  const double *C = B.Z + mv.mo, *eig = B.eig + mv.o0, *fill = B.fill + mv.o0;
  double *D = B.T + mv.mo, *W = B.A + mv.mo;
  const size_t nn = (size_t)n * n;
  if (k <= 0) {
    for (size_t idx = t; idx < nn; idx += bd) W[idx] = 0.0;
    return;
  }
  for (size_t idx = t; idx < (size_t)n * k; idx += bd) {
    const int j = (int)(idx / n);
    D[idx] = C[idx] * (fill[j] * eig[j]);
  }
  __syncthreads();
  cta_gemm<double, double>(n, n, k, 1.0, D, n, false, C, n, true, 0.0, W, n, kGLowerC, As, Bs);
  for (size_t idx = t; idx < nn; idx += bd) {
    const int i = (int)(idx % n), j = (int)(idx / n);
    if (i < j) W[idx] = W[j + (size_t)i * n];
  }
}

// Band term of the gradient per atom pair (i < j) of each molecule: central-difference SK block
// derivatives (forces.F90:548-669, nonscc.F90:428-484, delta = 2^-13) contracted with rho, W and the
// potential shift; the contribution to atom i is stored (atom j receives its negative). One CTA of
// four warps per molecule, one warp per pair; every pair is evaluated once.
__global__ void __launch_bounds__(128) batch_pair_grad_kernel(ModelDev M, BatchDev B) {
  __shared__ WarpSk ws_all[4][6];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int id = B.order[blockIdx.x];
  if (B.st[id].status != 0) return;
  const MolV mv = mol_view(B, id);
  const int n = mv.n, nat = mv.nat;
  const double *rho = B.rho + mv.mo, *W = B.A + mv.mo, *Vo = B.Vout + mv.a0;
  double *dp = B.dpair + 3 * B.pair_off[id];
  const double delta = 1.220703125e-4;
  const double inv2d = 1.0 / (2.0 * delta);
  for (int l1 = 0; l1 < nat; ++l1) {
    for (int l2 = l1 + 1 + w; l2 < nat; l2 += 4) {
      const long long p = (long long)l1 * (2 * nat - l1 - 1) / 2 + (l2 - l1 - 1);
      const int a1 = mv.a0 + l1, a2 = mv.a0 + l2;
      const int s1 = B.species[a1], s2 = B.species[a2];
      const double bx = B.xyz[3 * a2] - B.xyz[3 * a1];
      const double by = B.xyz[3 * a2 + 1] - B.xyz[3 * a1 + 1];
      const double bz = B.xyz[3 * a2 + 2] - B.xyz[3 * a1 + 2];
      const PairDev &P = M.pair[s1 * M.nsp + s2];
      if (bx * bx + by * by + bz * bz > P.sk_cut * P.sk_cut) {
        if (lane < 3) dp[3 * p + lane] = 0.0;
        continue;
      }
      for (int kq = 0; kq < 3; ++kq)
        for (int ii = 0; ii < 2; ++ii) {
          double v[3] = {bx, by, bz};
          v[kq] -= (double)(2 * (ii + 1) - 3) * delta;
          eval_blocks(M, s1, s2, v[0], v[1], v[2], ws_all[w][kq * 2 + ii], lane);
        }
      const int o1 = B.a_orb[a1] - mv.o0, o2 = B.a_orb[a2] - mv.o0;
      const int n1 = M.sp[s1].n_orb, n2 = M.sp[s2].n_orb;
      const double vs = 0.5 * (Vo[l1] + Vo[l2]);
      double dt[3] = {0.0, 0.0, 0.0};
      for (int idx = lane; idx < n1 * n2; idx += 32) {
        const int bb = idx % n2, aa = idx / n2;
        const double rv = rho[(o2 + bb) + (size_t)(o1 + aa) * n];
        const double wv = W[(o2 + bb) + (size_t)(o1 + aa) * n];
#pragma unroll
        for (int kq = 0; kq < 3; ++kq) {
          const double dh = (ws_all[w][2 * kq + 1].blk[0][bb][aa] - ws_all[w][2 * kq].blk[0][bb][aa]) * inv2d;
          const double ds = (ws_all[w][2 * kq + 1].blk[1][bb][aa] - ws_all[w][2 * kq].blk[1][bb][aa]) * inv2d;
          dt[kq] += 2.0 * (rv * dh - wv * ds) + 2.0 * vs * ds * rv;
        }
      }
      const double gx = warp_sum(dt[0]), gy = warp_sum(dt[1]), gz = warp_sum(dt[2]);
      if (lane == 0) {
        dp[3 * p] = gx;
        dp[3 * p + 1] = gy;
        dp[3 * p + 2] = gz;
      }
      __syncwarp();
    }
  }
}

// Gradient of every atom: the band terms of its pairs (summed in partner order, deterministic),
// SCC double counting (shortgamma.F90:349-411, coulomb.F90:1140-1185) and repulsive
// (twobodyrep.F90:273-332), partners restricted to the atom's molecule. One warp per atom.
__global__ void __launch_bounds__(64) batch_grad_kernel(ModelDev M, BatchDev B) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gA = blockIdx.x * 2 + w;
  if (gA >= B.natom) return;
  const int id = B.a_mol[gA];
  if (B.st[id].status != 0) {
    if (lane == 0) B.grad[3 * gA] = B.grad[3 * gA + 1] = B.grad[3 * gA + 2] = 0.0;
    return;
  }
  const MolV mv = mol_view(B, id);
  const int nat = mv.nat, a = gA - mv.a0;
  const double *dp = B.dpair + 3 * B.pair_off[id];
  double gx = 0.0, gy = 0.0, gz = 0.0;
  if (lane == 0) {
    for (int b = 0; b < nat; ++b) {
      if (b == a) continue;
      const int l1 = min(a, b), l2 = max(a, b);
      const long long p = (long long)l1 * (2 * nat - l1 - 1) / 2 + (l2 - l1 - 1);
      const double sgn = (a == l1) ? 1.0 : -1.0;
      gx += sgn * dp[3 * p];
      gy += sgn * dp[3 * p + 1];
      gz += sgn * dp[3 * p + 2];
    }
  }
  // double counting + repulsive
  const int sa = B.species[gA];
  const double ua = M.sp[sa].hubbu;
  const double dqa = B.qout[gA] - B.q0[gA];
  double hx = 0.0, hy = 0.0, hz = 0.0;
  for (int b = lane; b < mv.nat; b += 32) {
    if (b == a) continue;
    const int gb = mv.a0 + b;
    const int sb = B.species[gb];
    const double dx = B.xyz[3 * gA] - B.xyz[3 * gb], dy = B.xyz[3 * gA + 1] - B.xyz[3 * gb + 1],
                 dz = B.xyz[3 * gA + 2] - B.xyz[3 * gb + 2];
    const double r2 = dx * dx + dy * dy + dz * dz, r = sqrt(r2);
    const double qq = dqa * (B.qout[gb] - B.q0[gb]);
    double f = -qq / (r2 * r);
    const double rc = M.pair[sa * M.nsp + sb].gamma_cut;
    if (r2 <= rc * rc + kTolSameDist * kTolSameDist) f -= qq * exp_gamma_prime(r, M.sp[sb].hubbu, ua) / r;
    const PairDev &P = M.pair[sb * M.nsp + sa];
    if (r2 <= P.rep_cut * P.rep_cut) {
      double e, de;
      spline_rep(M.rep + P.off_rep, P.n_spline, r, &e, &de);
      f += de / r;
    }
    hx += f * dx;
    hy += f * dy;
    hz += f * dz;
  }
  hx = warp_sum(hx);
  hy = warp_sum(hy);
  hz = warp_sum(hz);
  if (lane == 0) {
    B.grad[3 * gA] = gx + hx;
    B.grad[3 * gA + 1] = gy + hy;
    B.grad[3 * gA + 2] = gz + hz;
  }
}

// ------------------------------------------------------------------------------ host drivers
namespace {

int fail(char *msg, size_t len, int code, const char *text) {
  if (msg && len) {
    std::strncpy(msg, text, len - 1);
    msg[len - 1] = '\0';
  }
  return code;
}

template <typename T>
int balloc(BatchState &b, T **p, size_t count, std::vector<void *> &owner) {
  *p = nullptr;
  if (count == 0) count = 1;
  if (cudaMalloc((void **)p, count * sizeof(T)) != cudaSuccess) return -1;
  owner.push_back(*p);
  return 0;
}

void free_list(std::vector<void *> &v) {
  for (void *p : v) cudaFree(p);
  v.clear();
}

}  // namespace

void batch_free(BatchState &b) {
  free_list(b.owned);
  free_list(b.bro_owned);
  if (b.h_active) cudaFreeHost(b.h_active);
  if (b.graph) cudaGraphExecDestroy(b.graph);
  b.graph = nullptr;
  b = BatchState{};
}

int batch_set_geometries(cudaStream_t s, BatchState &b, const ModelDev &m, const std::vector<SpeciesDev> &h_sp,
                         double cutoff, int nmol, const int *atom_off, const double *coords, const int *species,
                         bool coords_on_device, char *msg, size_t len) {
  if (nmol < 1 || !atom_off || !coords || !species) return fail(msg, len, DFTBGPU_ERR_ARGS, "batch: bad arguments");
  if (atom_off[0] != 0) return fail(msg, len, DFTBGPU_ERR_ARGS, "batch: atom_off[0] must be 0");
  const int natom = atom_off[nmol];
  std::vector<int> orb_off(nmol + 1, 0), a_orb(natom), a_mol(natom), o_atom;
  std::vector<long long> mat_off(nmol + 1, 0), gam_off(nmol + 1, 0), pair_off(nmol + 1, 0);
  char buf[256];
  for (int i = 0; i < nmol; ++i) {
    const int na = atom_off[i + 1] - atom_off[i];
    if (na < 1 || na > kBatchMaxAtom) {
      std::snprintf(buf, sizeof(buf), "batch: molecule %d has %d atoms (1..%d supported)", i, na, kBatchMaxAtom);
      return fail(msg, len, DFTBGPU_ERR_ARGS, buf);
    }
    int no = 0;
    for (int a = atom_off[i]; a < atom_off[i + 1]; ++a) {
      const int sp = species[a];
      if (sp < 0 || sp >= (int)h_sp.size()) {
        std::snprintf(buf, sizeof(buf), "batch: atom %d: species %d out of range", a, sp);
        return fail(msg, len, DFTBGPU_ERR_ARGS, buf);
      }
      a_orb[a] = orb_off[i] + no;
      a_mol[a] = i;
      for (int q = 0; q < h_sp[sp].n_orb; ++q) o_atom.push_back(a);
      no += h_sp[sp].n_orb;
    }
    if (no > kBatchMaxOrb) {
      std::snprintf(buf, sizeof(buf), "batch: molecule %d has %d orbitals (at most %d)", i, no, kBatchMaxOrb);
      return fail(msg, len, DFTBGPU_ERR_ARGS, buf);
    }
    orb_off[i + 1] = orb_off[i] + no;
    mat_off[i + 1] = mat_off[i] + (long long)no * no;
    gam_off[i + 1] = gam_off[i] + (long long)na * na;
    pair_off[i + 1] = pair_off[i] + (long long)na * (na - 1) / 2;
  }
  const int norb = orb_off[nmol];
  std::vector<int> order(nmol);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return orb_off[x + 1] - orb_off[x] > orb_off[y + 1] - orb_off[y];
  });
  const bool grow = (size_t)nmol > b.cap_mol || (size_t)natom > b.cap_atom || (size_t)norb > b.cap_orb ||
                    (size_t)mat_off[nmol] > b.cap_mat || (size_t)gam_off[nmol] > b.cap_gam ||
                    (size_t)pair_off[nmol] > b.cap_pair;
  BatchDev &d = b.d;
  if (grow) {
    free_list(b.owned);
    free_list(b.bro_owned);
    b.cap_M = 0;
    const size_t NM = nmol, NA = natom, NO = norb, MM = mat_off[nmol], NG = gam_off[nmol];
    int e = 0;
    int *ip;
    long long *lp;
    e |= balloc(b, &ip, NM + 1, b.owned); d.atom_off = ip;
    e |= balloc(b, &ip, NM + 1, b.owned); d.orb_off = ip;
    e |= balloc(b, &lp, NM + 1, b.owned); d.mat_off = lp;
    e |= balloc(b, &lp, NM + 1, b.owned); d.gam_off = lp;
    e |= balloc(b, &lp, NM + 1, b.owned); d.pair_off = lp;
    e |= balloc(b, &d.dpair, 3 * (size_t)std::max(pair_off[nmol], 1LL), b.owned);
    e |= balloc(b, &ip, NM, b.owned); d.order = ip;
    e |= balloc(b, &ip, NA, b.owned); d.a_orb = ip;
    e |= balloc(b, &ip, NA, b.owned); d.a_mol = ip;
    e |= balloc(b, &ip, NA, b.owned); d.species = ip;
    e |= balloc(b, &ip, NO, b.owned); d.o_atom = ip;
    double *dp;
    e |= balloc(b, &dp, 3 * NA, b.owned); d.xyz = dp;
    for (double **pp : {&d.q0, &d.qin, &d.qout, &d.V, &d.Vout, &d.erep, &d.qlast, &d.dlast})
      e |= balloc(b, pp, NA, b.owned);
    e |= balloc(b, &d.grad, 3 * NA, b.owned);
    for (double **pp : {&d.eig, &d.fill, &d.dd, &d.ee}) e |= balloc(b, pp, NO, b.owned);
    for (double **pp : {&d.H0, &d.S, &d.L, &d.Li, &d.A0, &d.A, &d.T, &d.Z, &d.rho}) e |= balloc(b, pp, MM, b.owned);
    for (float **pp : {&d.L32, &d.Li32, &d.A0_32, &d.A32, &d.T32, &d.Z32, &d.X32, &d.C32, &d.Mt32, &d.Zp32})
      e |= balloc(b, pp, MM, b.owned);
    e |= balloc(b, &d.rho_ref, MM, b.owned);
    e |= balloc(b, &d.Vref, NA, b.owned);
    e |= balloc(b, &d.gam, NG, b.owned);
    e |= balloc(b, &d.st, NM, b.owned);
    e |= balloc(b, &b.d_active, 1, b.owned);
    if (e) {
      free_list(b.owned);
      b.cap_mol = b.cap_atom = b.cap_orb = b.cap_mat = b.cap_gam = b.cap_pair = 0;
      return fail(msg, len, DFTBGPU_ERR_CUDA, "batch: device allocation failed");
    }
    b.cap_mol = NM;
    b.cap_atom = NA;
    b.cap_orb = NO;
    b.cap_mat = MM;
    b.cap_gam = NG;
    b.cap_pair = (size_t)pair_off[nmol];
  }
  b.nmol = d.nmol = nmol;
  b.natom = d.natom = natom;
  b.norb = d.norb = norb;
  b.nmat = mat_off[nmol];
  b.ngam = gam_off[nmol];
  b.h_atom_off.assign(atom_off, atom_off + nmol + 1);
  b.h_orb_off = orb_off;
  b.h_mat_off = mat_off;
  b.h_species.assign(species, species + natom);
  auto up = [&](const void *dst, const void *src, size_t bytes) {
    return cudaMemcpyAsync(const_cast<void *>(dst), src, bytes, cudaMemcpyHostToDevice, s);
  };
  cudaError_t ce = cudaSuccess;
  auto acc = [&](cudaError_t x) { if (x != cudaSuccess) ce = x; };
  acc(up(d.atom_off, atom_off, sizeof(int) * (nmol + 1)));
  acc(up(d.orb_off, orb_off.data(), sizeof(int) * (nmol + 1)));
  acc(up(d.mat_off, mat_off.data(), sizeof(long long) * (nmol + 1)));
  acc(up(d.gam_off, gam_off.data(), sizeof(long long) * (nmol + 1)));
  acc(up(d.pair_off, pair_off.data(), sizeof(long long) * (nmol + 1)));
  acc(up(d.order, order.data(), sizeof(int) * nmol));
  acc(up(d.a_orb, a_orb.data(), sizeof(int) * natom));
  acc(up(d.a_mol, a_mol.data(), sizeof(int) * natom));
  acc(up(d.species, species, sizeof(int) * natom));
  acc(up(d.o_atom, o_atom.data(), sizeof(int) * norb));
  acc(cudaMemcpyAsync(const_cast<double *>(d.xyz), coords, sizeof(double) * 3 * natom,
                      coords_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  if (ce != cudaSuccess) return fail(msg, len, DFTBGPU_ERR_CUDA, cudaGetErrorString(ce));
  batch_geom_kernel<<<nmol, kBatchThreads, 0, s>>>(m, d, cutoff * cutoff);
  count_launch();
  acc(cudaGetLastError());
  std::vector<MolState> hst(nmol);
  acc(cudaMemcpyAsync(hst.data(), d.st, sizeof(MolState) * nmol, cudaMemcpyDeviceToHost, s));
  acc(cudaStreamSynchronize(s));
  if (ce != cudaSuccess) return fail(msg, len, DFTBGPU_ERR_CUDA, cudaGetErrorString(ce));
  b.have_geom = true;
  b.have_scc = false;
  for (int i = 0; i < nmol; ++i)
    if (hst[i].status == kDevNotPosDef) {
      std::snprintf(buf, sizeof(buf), "batch: molecule %d: overlap matrix is not positive definite", i);
      return fail(msg, len, DFTBGPU_ERR_NOT_POSDEF, buf);
    }
  return DFTBGPU_OK;
}

int batch_scc(cudaStream_t s, BatchState &b, const ModelDev &m, const BatchOpts &o, char *msg, size_t len) {
  if (!b.have_geom) return fail(msg, len, DFTBGPU_ERR_STATE, "batch: no geometries set");
  BatchDev &d = b.d;
  if ((size_t)o.max_iter > b.cap_M) {
    free_list(b.bro_owned);
    const size_t NM = b.cap_mol, NA = b.cap_atom, M = (size_t)o.max_iter;
    int e = 0;
    e |= balloc(b, &d.ww, NM * M, b.bro_owned);
    e |= balloc(b, &d.cc, NM * M, b.bro_owned);
    e |= balloc(b, &d.aa, NM * M * M, b.bro_owned);
    e |= balloc(b, &d.beta, NM * M * M, b.bro_owned);
    e |= balloc(b, &d.dF, NA * M, b.bro_owned);
    e |= balloc(b, &d.uu, NA * M, b.bro_owned);
    if (e) {
      free_list(b.bro_owned);
      b.cap_M = 0;
      return fail(msg, len, DFTBGPU_ERR_CUDA, "batch: device allocation failed (Broyden history)");
    }
    b.cap_M = M;
  }
  d.M = (int)b.cap_M;
  if (!b.h_active && cudaHostAlloc((void **)&b.h_active, sizeof(int), cudaHostAllocDefault) != cudaSuccess)
    return fail(msg, len, DFTBGPU_ERR_CUDA, "batch: pinned allocation failed");
  int nmax = 1;
  for (int i = 0; i < b.nmol; ++i) nmax = std::max(nmax, b.h_orb_off[i + 1] - b.h_orb_off[i]);
  const size_t sm64 = 4 * (size_t)nmax * sizeof(double) + (size_t)nmax * sizeof(int);
  const size_t sm32 = 4 * (size_t)nmax * sizeof(float) + (size_t)nmax * sizeof(int);
  batch_scc_init_kernel<<<b.nmol, kBatchThreads, 0, s>>>(d, o);
  count_launch();
  // one SCC iteration of all molecules as a CUDA graph: reset the active count, the FP64 iteration
  // kernel, the FP32 one (mixed form), read the count back
  cudaGraph_t g = nullptr;
  cudaError_t ce = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (ce == cudaSuccess) {
    cudaMemsetAsync(b.d_active, 0, sizeof(int), s);
    batch_iter_kernel<double><<<b.nmol, kBatchThreads, sm64, s>>>(m, d, o, b.d_active);
    if (o.mixed) {
      batch_iter_kernel<float><<<b.nmol, kBatchThreads, sm32, s>>>(m, d, o, b.d_active);
      batch_pert_kernel<<<b.nmol, kBatchThreads, 0, s>>>(m, d, o, b.d_active);
    }
    cudaMemcpyAsync(b.h_active, b.d_active, sizeof(int), cudaMemcpyDeviceToHost, s);
    ce = cudaStreamEndCapture(s, &g);
  }
  if (ce != cudaSuccess) return fail(msg, len, DFTBGPU_ERR_CUDA, cudaGetErrorString(ce));
  if (b.graph) cudaGraphExecDestroy(b.graph);
  b.graph = nullptr;
  ce = cudaGraphInstantiate(&b.graph, g, 0);
  cudaGraphDestroy(g);
  if (ce != cudaSuccess) return fail(msg, len, DFTBGPU_ERR_CUDA, cudaGetErrorString(ce));
  for (int it = 0; it <= o.max_iter; ++it) {
    ce = cudaGraphLaunch(b.graph, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) return fail(msg, len, DFTBGPU_ERR_CUDA, cudaGetErrorString(ce));
    count_launch(o.mixed ? 3 : 1);
    if (*b.h_active == 0) break;
  }
  b.have_scc = true;
  b.have_w = false;
  return DFTBGPU_OK;
}

int batch_gradients(cudaStream_t s, BatchState &b, const ModelDev &m, char *msg, size_t len) {
  if (!b.have_scc) return fail(msg, len, DFTBGPU_ERR_STATE, "batch: call the batched SCC first");
  batch_ew_kernel<<<b.nmol, kBatchThreads, 0, s>>>(b.d);
  batch_pair_grad_kernel<<<b.nmol, 128, 0, s>>>(m, b.d);
  batch_grad_kernel<<<(b.natom + 1) / 2, 64, 0, s>>>(m, b.d);
  count_launch(3);
  b.have_w = true;
  const cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return fail(msg, len, DFTBGPU_ERR_CUDA, cudaGetErrorString(ce));
  return DFTBGPU_OK;
}

}  // namespace dg
