// FP64 dense kernels: GEMM with triangular skipping, blocked Cholesky, triangular inverse,
// blocked Householder tridiagonalisation (lower) and its back-transformation.
//
// These replace the LAPACK/MAGMA calls behind hegvd/magmaHegvd (math/eigensolver.F90:561-660,
// :1143-1245): potrf + sygst are expressed as a Cholesky factor L, its inverse X = L^-1 and two
// GEMMs (A = X H X^T), sytrd/ormtr as below, the tridiagonal solve lives in stedc.cu.
#include <cmath>
#include <type_traits>

#include "gridsync.cuh"
#include "linalg.cuh"

namespace dg {

// ------------------------------------------------------------------------------------- GEMM
// 64x64 output tile per CTA, 256 threads, 4x4 outputs per thread (strided by 16 so that shared
// memory reads are conflict-free), K step 16, register prefetch of the next K slab.
// With P != nullptr the CTA (x, y, z) sums only the z-th of gridDim.z slices of its k-range and
// writes the raw sum to P + z*m*n (split-K; dgemm_splitk_reduce applies alpha/beta in a fixed
// order, so results stay deterministic).
template <typename T, bool TA, bool TB>
__global__ void __launch_bounds__(256) dgemm_kernel(int m, int n, int k, T alpha,
                                                    const T *__restrict__ A, int lda,
                                                    const T *__restrict__ B, int ldb,
                                                    T beta, T *__restrict__ C, int ldc,
                                                    int flags, T *__restrict__ P) {
  constexpr int BM = 64, BN = 64, BK = 16;
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int i0 = blockIdx.x * BM, j0 = blockIdx.y * BN;
  if ((flags & kCLower) && i0 + BM - 1 < j0) return;
  int kmin = 0, kmax = k;
  if (flags & kALower) kmax = min(kmax, i0 + BM);
  if (flags & kAUpper) kmin = max(kmin, i0);
  if (flags & kBLower) kmin = max(kmin, j0);
  if (flags & kBUpper) kmax = min(kmax, j0 + BN);
  if (P != nullptr && gridDim.z > 1) {
    int span = max(kmax - kmin, 0);
    int chunk = ((span + gridDim.z - 1) / gridDim.z + BK - 1) / BK * BK;
    int lo = kmin + blockIdx.z * chunk;
    kmax = min(kmax, lo + chunk);
    kmin = lo;
  }

  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = T(0);

  T ra[4], rb[4];
  auto load_a = [&](int p0) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      int t = tid + 256 * r;
      int ii, pp;
      if (!TA) { ii = t & 63; pp = t >> 6; } else { pp = t & 15; ii = t >> 4; }
      int gi = i0 + ii, gp = p0 + pp;
      T v = T(0);
      if (gi < m && gp < kmax) v = TA ? A[gp + (size_t)gi * lda] : A[gi + (size_t)gp * lda];
      ra[r] = v;
    }
  };
  auto load_b = [&](int p0) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      int t = tid + 256 * r;
      int pp, jj;
      if (!TB) { pp = t & 15; jj = t >> 4; } else { jj = t & 63; pp = t >> 6; }
      int gj = j0 + jj, gp = p0 + pp;
      T v = T(0);
      if (gj < n && gp < kmax) v = TB ? B[gj + (size_t)gp * ldb] : B[gp + (size_t)gj * ldb];
      rb[r] = v;
    }
  };
  auto store_ab = [&]() {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      int t = tid + 256 * r;
      int ii, pp;
      if (!TA) { ii = t & 63; pp = t >> 6; } else { pp = t & 15; ii = t >> 4; }
      As[pp][ii] = ra[r];
      int jj, qq;
      if (!TB) { qq = t & 15; jj = t >> 4; } else { jj = t & 63; qq = t >> 6; }
      Bs[qq][jj] = rb[r];
    }
  };

  if (kmin < kmax) {
    load_a(kmin);
    load_b(kmin);
    for (int p0 = kmin; p0 < kmax; p0 += BK) {
      __syncthreads();
      store_ab();
      __syncthreads();
      if (p0 + BK < kmax) {
        load_a(p0 + BK);
        load_b(p0 + BK);
      }
#pragma unroll
      for (int pp = 0; pp < BK; ++pp) {
        T a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = As[pp][tx + 16 * i];
#pragma unroll
        for (int j = 0; j < 4; ++j) b[j] = Bs[pp][ty + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
      }
    }
  }
  if (P != nullptr) {
    T *Pz = P + (size_t)blockIdx.z * m * n;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      int gi = i0 + tx + 16 * i;
      if (gi >= m) continue;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        int gj = j0 + ty + 16 * j;
        if (gj < n) Pz[gi + (size_t)gj * m] = acc[i][j];
      }
    }
    return;
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int gi = i0 + tx + 16 * i;
    if (gi >= m) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int gj = j0 + ty + 16 * j;
      if (gj >= n) continue;
      T *c = C + gi + (size_t)gj * ldc;
      T v = alpha * acc[i][j];
      if (beta != T(0)) v = fma(beta, *c, v);
      *c = v;
    }
  }
}

// C = alpha * sum_z P[z] + beta * C over the tiles a split-K dgemm computed.
template <typename T>
__global__ void dgemm_splitk_reduce(int m, int n, int splits, const T *__restrict__ P, T alpha,
                                    T beta, T *__restrict__ C, int ldc, int flags) {
  size_t total = (size_t)m * n;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(idx % m), j = (int)(idx / m);
    if ((flags & kCLower) && (i | 63) < (j & ~63)) continue;  // tile skipped by the GEMM
    T s = T(0);
    for (int z = 0; z < splits; ++z) s += P[(size_t)z * total + idx];
    T *c = C + i + (size_t)j * ldc;
    T v = alpha * s;
    if (beta != T(0)) v = fma(beta, *c, v);
    *c = v;
  }
}

// FP32 GEMM for products with many output tiles: 128 x 128 tile per CTA, 256 threads, 8 x 8 outputs
// per thread (rows tx*4 + {0..3} and 64 + tx*4 + {0..3}, columns likewise from ty, so that shared
// memory is read as float4 without bank conflicts), K step 16 with register prefetch of the next
// slab. Shared rows are padded to 132 floats so that the transposed stores of either operand layout
// are conflict-free. Same flags as dgemm_kernel; with kCLower only elements on or below the diagonal
// are written. No split-K (it is used only where the tiles fill the GPU). Two CTAs per SM (128
// registers per thread).
template <bool TA, bool TB>
__global__ void __launch_bounds__(256, 2) sgemm128_kernel(int m, int n, int k, float alpha,
                                                      const float *__restrict__ A, int lda,
                                                      const float *__restrict__ B, int ldb, float beta,
                                                      float *__restrict__ C, int ldc, int flags) {
  constexpr int BM = 128, BN = 128, BK = 16, LDS = 132;
  __shared__ __align__(16) float As[BK][LDS];
  __shared__ __align__(16) float Bs[BK][LDS];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int i0 = blockIdx.x * BM, j0 = blockIdx.y * BN;
  if ((flags & kCLower) && i0 + BM - 1 < j0) return;
  int kmin = 0, kmax = k;
  if (flags & kALower) kmax = min(kmax, i0 + BM);
  if (flags & kAUpper) kmin = max(kmin, i0);
  if (flags & kBLower) kmin = max(kmin, j0);
  if (flags & kBUpper) kmax = min(kmax, j0 + BN);

  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;

  float ra[8], rb[8];
  // element q of this thread's share of a 128 x 16 slab: (row, kk) with the contiguous source index
  // running fastest across threads
  auto load_a = [&](int p0) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int t = tid + 256 * q;
      int ii, pp;
      if (!TA) { ii = t & 127; pp = t >> 7; } else { pp = t & 15; ii = t >> 4; }
      const int gi = i0 + ii, gp = p0 + pp;
      float v = 0.f;
      if (gi < m && gp < kmax) v = TA ? A[gp + (size_t)gi * lda] : A[gi + (size_t)gp * lda];
      ra[q] = v;
    }
  };
  auto load_b = [&](int p0) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int t = tid + 256 * q;
      int jj, pp;
      if (TB) { jj = t & 127; pp = t >> 7; } else { pp = t & 15; jj = t >> 4; }
      const int gj = j0 + jj, gp = p0 + pp;
      float v = 0.f;
      if (gj < n && gp < kmax) v = TB ? B[gj + (size_t)gp * ldb] : B[gp + (size_t)gj * ldb];
      rb[q] = v;
    }
  };
  auto store_ab = [&]() {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int t = tid + 256 * q;
      int ii, pp;
      if (!TA) { ii = t & 127; pp = t >> 7; } else { pp = t & 15; ii = t >> 4; }
      As[pp][ii] = ra[q];
      int jj, qq;
      if (TB) { jj = t & 127; qq = t >> 7; } else { qq = t & 15; jj = t >> 4; }
      Bs[qq][jj] = rb[q];
    }
  };

  if (kmin < kmax) {
    load_a(kmin);
    load_b(kmin);
    for (int p0 = kmin; p0 < kmax; p0 += BK) {
      __syncthreads();
      store_ab();
      __syncthreads();
      if (p0 + BK < kmax) {
        load_a(p0 + BK);
        load_b(p0 + BK);
      }
#pragma unroll
      for (int pp = 0; pp < BK; ++pp) {
        const float4 a0 = *reinterpret_cast<const float4 *>(&As[pp][tx * 4]);
        const float4 a1 = *reinterpret_cast<const float4 *>(&As[pp][64 + tx * 4]);
        const float4 b0 = *reinterpret_cast<const float4 *>(&Bs[pp][ty * 4]);
        const float4 b1 = *reinterpret_cast<const float4 *>(&Bs[pp][64 + ty * 4]);
        const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
        const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
          for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
      }
    }
  }
  const bool lower = (flags & kCLower) != 0;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int gj = j0 + (j < 4 ? ty * 4 + j : 64 + ty * 4 + (j - 4));
    if (gj >= n) continue;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int gi = i0 + (i < 4 ? tx * 4 + i : 64 + tx * 4 + (i - 4));
      if (gi >= m || (lower && gi < gj)) continue;
      float *c = C + gi + (size_t)gj * ldc;
      float v = alpha * acc[i][j];
      if (beta != 0.f) v = fmaf(beta, *c, v);
      *c = v;
    }
  }
}

std::atomic<bool> g_sgemm128{true};   // FP32 products with many tiles on sgemm128_kernel
std::atomic<int> g_panel_mode{1};

thread_local GemmProfile g_gemm_prof;

static double gemm_executed_flops(int m, int n, int k, int flags) {
  double f = 0.0;
  for (int i0 = 0; i0 < m; i0 += 64)
    for (int j0 = 0; j0 < n; j0 += 64) {
      if ((flags & kCLower) && i0 + 63 < j0) continue;
      int kmin = 0, kmax = k;
      if (flags & kALower) kmax = std::min(kmax, i0 + 64);
      if (flags & kAUpper) kmin = std::max(kmin, i0);
      if (flags & kBLower) kmin = std::max(kmin, j0);
      if (flags & kBUpper) kmax = std::min(kmax, j0 + 64);
      if (kmax > kmin) f += 2.0 * std::min(64, m - i0) * std::min(64, n - j0) * (double)(kmax - kmin);
    }
  return f;
}

// The digit-slice product runs one 128 x 64 tile per SM at about 5 us per 64-wide K block (split
// along K when it has few tiles); FP64 FMA runs about 6e11 multiply-adds/s over the whole GPU. Route a
// product to the tensor cores only where that estimate says it is faster.
static bool tc_dgemm_faster(int m, int n, int k) {
  return tc_dgemm_estimate_s(m, n, k) < (double)m * n * k / 6e11;
}

template <typename T>
void gemm(cudaStream_t s, char ta, char tb, int m, int n, int k, T alpha, const T *A, int lda, const T *B,
          int ldb, T beta, T *C, int ldc, int flags, T *work, size_t work_elems) {
  if (m <= 0 || n <= 0) return;
  dim3 grid(ceil_div(m, 64), ceil_div(n, 64));
  bool TA = (ta == 'T' || ta == 't'), TB = (tb == 'T' || tb == 't');
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(s, &cap);
  const bool prof = g_gemm_prof.on && cap == cudaStreamCaptureStatusNone;
  if (prof) {
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
  }
  // Split-K when the output has too few tiles to fill the GPU and K is long.
  int splits = 1;
  long long tiles = (long long)grid.x * grid.y;
  if (work && tiles < kSplitTarget && k >= 1024) {
    long long sp = (kSplitTarget + tiles - 1) / tiles;
    sp = std::min(sp, (long long)k / 256);
    sp = std::min(sp, 64LL);
    sp = std::min(sp, (long long)(work_elems / ((size_t)m * n)));
    splits = (int)sp;
    if (splits < 2) splits = 1;
  }
  T *P = (splits > 1) ? work : nullptr;
  grid.z = splits;
  bool done = false, on_tc = false;
  if constexpr (std::is_same<T, double>::value) {
    if (g_tc_dgemm && m >= 64 && n >= 64 && k >= 32 && cap == cudaStreamCaptureStatusNone &&
        tc_dgemm_faster(m, n, k)) {
      // a scratch allocation that fails leaves the product to the FP64 FMA kernel below
      if (tc_dgemm(s, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, flags) == 0) {
        done = true;
        on_tc = true;
        P = nullptr;
      }
    }
  }
  if constexpr (std::is_same<T, float>::value) {
    if (g_tc_fgemm && m >= 512 && n >= 512 && k >= 512 && cap == cudaStreamCaptureStatusNone) {
      // a scratch allocation that fails leaves the product to the FP32 FMA kernels below
      if (tc_fgemm(s, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, flags) == 0) {
        done = true;
        P = nullptr;
      }
    }
    const long long tiles128 = (long long)ceil_div(m, 128) * ceil_div(n, 128);
    if (!done && g_sgemm128 && tiles128 >= 2 * 152) {
      const dim3 g128(ceil_div(m, 128), ceil_div(n, 128));
      if (!TA && !TB)
        sgemm128_kernel<false, false><<<g128, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, flags);
      else if (!TA && TB)
        sgemm128_kernel<false, true><<<g128, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, flags);
      else if (TA && !TB)
        sgemm128_kernel<true, false><<<g128, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, flags);
      else
        sgemm128_kernel<true, true><<<g128, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, flags);
      count_launch();
      done = true;
      P = nullptr;
    }
  }
  if (done) {
  } else if (!TA && !TB)
    dgemm_kernel<T, false, false><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, flags, P);
  else if (!TA && TB)
    dgemm_kernel<T, false, true><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, flags, P);
  else if (TA && !TB)
    dgemm_kernel<T, true, false><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, flags, P);
  else
    dgemm_kernel<T, true, true><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, flags, P);
  if (!done) count_launch();
  if (P) {
    int rb = (int)std::min<long long>(((long long)m * n + 255) / 256, 152 * 8);
    dgemm_splitk_reduce<T><<<rb, 256, 0, s>>>(m, n, splits, P, alpha, beta, C, ldc, flags);
    count_launch();
  }
  if (prof) {
    cudaEventRecord(e1, s);
    g_gemm_prof.ev.push_back(e0);
    g_gemm_prof.ev.push_back(e1);
    g_gemm_prof.flops.push_back(gemm_executed_flops(m, n, k, flags));
    g_gemm_prof.phase.push_back(on_tc ? kPhGemmTc : (sizeof(T) == 4 ? kPhGemm32 : kPhGemm));
  }
}

template void gemm<double>(cudaStream_t, char, char, int, int, int, double, const double *, int,
                           const double *, int, double, double *, int, int, double *, size_t);
template void gemm<float>(cudaStream_t, char, char, int, int, int, float, const float *, int, const float *,
                          int, float, float *, int, int, float *, size_t);

void dgemm(cudaStream_t s, char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda,
           const double *B, int ldb, double beta, double *C, int ldc, int flags, double *work,
           size_t work_elems) {
  gemm<double>(s, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, flags, work, work_elems);
}

// ------------------------------------------------------------------------------------- helpers
__global__ void set_zero_kernel(double *p, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    p[i] = 0.0;
}
void set_zero(cudaStream_t s, double *p, size_t n) {
  if (!n) return;
  int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
  set_zero_kernel<<<blocks, 256, 0, s>>>(p, n);
  count_launch();
}

// 32x32 tiles through shared memory so both the read (lower) and the write (upper) are coalesced.
template <typename T>
__global__ void lower_to_upper_kernel(int n, T *A, int lda) {
  __shared__ T t[32][33];
  int bi = blockIdx.x, bj = blockIdx.y;  // tile (bi, bj) with bi >= bj in the lower triangle
  if (bi < bj) return;
  int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int r = ty; r < 32; r += 8) {
    int gi = bi * 32 + tx, gj = bj * 32 + r;
    t[r][tx] = (gi < n && gj < n) ? A[gi + (size_t)gj * lda] : T(0);
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    int gi = bj * 32 + tx, gj = bi * 32 + r;   // write A(gi, gj) = A(gj, gi) for gj > gi
    if (gi < n && gj < n && gj > gi) A[gi + (size_t)gj * lda] = t[tx][r];
  }
}
template <typename T>
void copy_lower_to_upper(cudaStream_t s, int n, T *A, int lda) {
  dim3 g(ceil_div(n, 32), ceil_div(n, 32));
  lower_to_upper_kernel<T><<<g, dim3(32, 8), 0, s>>>(n, A, lda);
  count_launch();
}
template void copy_lower_to_upper<double>(cudaStream_t, int, double *, int);
template void copy_lower_to_upper<float>(cudaStream_t, int, float *, int);

__global__ void zero_upper_kernel(int n, double *A, int lda) {
  int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < j && i < n; i += gridDim.x * blockDim.x)
    A[i + (size_t)j * lda] = 0.0;
}
void zero_strict_upper(cudaStream_t s, int n, double *A, int lda) {
  dim3 g(ceil_div(n, 256), n);
  zero_upper_kernel<<<g, 256, 0, s>>>(n, A, lda);
  count_launch();
}

template <typename T>
__global__ void scale_columns_kernel(int m, int n, const T *A, int lda, const double *f, T *B, int ldb) {
  int j = blockIdx.y;
  T fj = (T)f[j];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
    B[i + (size_t)j * ldb] = A[i + (size_t)j * lda] * fj;
}
template <typename T>
void scale_columns(cudaStream_t s, int m, int n, const T *A, int lda, const double *f, T *B, int ldb) {
  if (m <= 0 || n <= 0) return;
  dim3 g(std::min(ceil_div(m, 256), 8), n);
  scale_columns_kernel<T><<<g, 256, 0, s>>>(m, n, A, lda, f, B, ldb);
  count_launch();
}
template void scale_columns<double>(cudaStream_t, int, int, const double *, int, const double *, double *, int);
template void scale_columns<float>(cudaStream_t, int, int, const float *, int, const double *, float *, int);

template <typename T>
__global__ void set_zero_t_kernel(T *p, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    p[i] = T(0);
}
template <typename T>
void set_zero_t(cudaStream_t s, T *p, size_t n) {
  if (!n) return;
  int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
  set_zero_t_kernel<T><<<blocks, 256, 0, s>>>(p, n);
  count_launch();
}
template void set_zero_t<float>(cudaStream_t, float *, size_t);
template void set_zero_t<double>(cudaStream_t, double *, size_t);

// ------------------------------------------------------------------------------------- Cholesky
constexpr int NB = 64;

// Unblocked Cholesky of one jb x jb diagonal block in shared memory.
__global__ void potf2_kernel(int jb, double *A, int lda, int *status) {
  __shared__ double a[NB][NB + 1];
  const int t = threadIdx.x;
  for (int idx = t; idx < jb * jb; idx += blockDim.x) {
    int r = idx % jb, c = idx / jb;
    a[r][c] = (r >= c) ? A[r + (size_t)c * lda] : 0.0;
  }
  __syncthreads();
  for (int c = 0; c < jb; ++c) {
    double piv = a[c][c];
    bool bad = !(piv > 0.0) || !isfinite(piv);
    if (bad && t == 0) atomicExch(status, kDevNotPosDef);
    double sq = sqrt(bad ? 1.0 : piv);
    __syncthreads();
    if (t == 0) a[c][c] = sq;
    for (int r = c + 1 + t; r < jb; r += blockDim.x) a[r][c] /= sq;
    __syncthreads();
    int mr = jb - c - 1;
    for (int idx = t; idx < mr * mr; idx += blockDim.x) {
      int r = c + 1 + idx % mr, q = c + 1 + idx / mr;
      if (r >= q) a[r][q] = fma(-a[r][c], a[q][c], a[r][q]);
    }
    __syncthreads();
  }
  for (int idx = t; idx < jb * jb; idx += blockDim.x) {
    int r = idx % jb, c = idx / jb;
    A[r + (size_t)c * lda] = (r >= c) ? a[r][c] : 0.0;
  }
}

// Solve X L11^T = B for the panel rows below the diagonal block (B overwritten by X).
__global__ void trsm_panel_kernel(int m, int jb, const double *L, int ldl, double *B, int ldb) {
  __shared__ double l[NB][NB + 1];
  __shared__ double x[NB][NB + 1];
  const int t = threadIdx.x;
  const int r0 = blockIdx.x * NB;
  for (int idx = t; idx < jb * jb; idx += blockDim.x) {
    int r = idx % jb, c = idx / jb;
    l[r][c] = (r >= c) ? L[r + (size_t)c * ldl] : 0.0;
  }
  for (int idx = t; idx < NB * jb; idx += blockDim.x) {
    int r = idx % NB, c = idx / NB;
    x[r][c] = (r0 + r < m) ? B[r0 + r + (size_t)c * ldb] : 0.0;
  }
  __syncthreads();
  if (t < NB && r0 + t < m) {
    for (int c = 0; c < jb; ++c) {
      double v = x[t][c];
      for (int q = 0; q < c; ++q) v = fma(-x[t][q], l[c][q], v);
      x[t][c] = v / l[c][c];
    }
  }
  __syncthreads();
  for (int idx = t; idx < NB * jb; idx += blockDim.x) {
    int r = idx % NB, c = idx / NB;
    if (r0 + r < m) B[r0 + r + (size_t)c * ldb] = x[r][c];
  }
}

void potrf_lower(cudaStream_t s, int n, double *A, int lda, int *status_dev) {
  for (int j0 = 0; j0 < n; j0 += NB) {
    int jb = std::min(NB, n - j0);
    double *Ajj = A + j0 + (size_t)j0 * lda;
    potf2_kernel<<<1, 256, 0, s>>>(jb, Ajj, lda, status_dev);
    count_launch();
    int m = n - j0 - jb;
    if (m > 0) {
      double *B = A + j0 + jb + (size_t)j0 * lda;
      trsm_panel_kernel<<<ceil_div(m, NB), 256, 0, s>>>(m, jb, Ajj, lda, B, lda);
      count_launch();
      double *A22 = A + j0 + jb + (size_t)(j0 + jb) * lda;
      dgemm(s, 'N', 'T', m, m, jb, -1.0, B, lda, B, lda, 1.0, A22, lda, kCLower);
    }
  }
  zero_strict_upper(s, n, A, lda);
}

// ------------------------------------------------------------------------------------- L^-1
__global__ void trtri_diag_kernel(int n, const double *L, int ldl, double *X, int ldx) {
  __shared__ double l[NB][NB + 1];
  __shared__ double x[NB][NB + 1];
  const int j0 = blockIdx.x * NB;
  const int jb = min(NB, n - j0);
  const int t = threadIdx.x;
  for (int idx = t; idx < jb * jb; idx += blockDim.x) {
    int r = idx % jb, c = idx / jb;
    l[r][c] = (r >= c) ? L[j0 + r + (size_t)(j0 + c) * ldl] : 0.0;
    x[r][c] = 0.0;
  }
  __syncthreads();
  if (t < jb) {
    for (int r = t; r < jb; ++r) {
      double v = (r == t) ? 1.0 : 0.0;
      for (int q = t; q < r; ++q) v = fma(-l[r][q], x[q][t], v);
      x[r][t] = v / l[r][r];
    }
  }
  __syncthreads();
  for (int idx = t; idx < jb * jb; idx += blockDim.x) {
    int r = idx % jb, c = idx / jb;
    X[j0 + r + (size_t)(j0 + c) * ldx] = x[r][c];
  }
}

// Off-diagonal blocks of X = L^-1 for the rows and columns [a, b), recursively: with the split h (a
// block boundary), X(h:b, a:h) = -X(h:b, h:b) L(h:b, a:h) X(a:h, a:h) once both diagonal halves are
// inverted. The two products are square-ish triangular GEMMs (n^3 / 3 FLOPs in all), which keeps
// them efficient on FP64 FMA and lets the tensor-core route take them where it is enabled.
static void trtri_rec(cudaStream_t s, int a, int b, const double *L, int ldl, double *X, int ldx, double *work,
                      size_t work_elems) {
  if (b - a <= NB) return;
  const int h = a + ceil_div(ceil_div(b - a, NB), 2) * NB;
  trtri_rec(s, a, h, L, ldl, X, ldx, work, work_elems);
  trtri_rec(s, h, b, L, ldl, X, ldx, work, work_elems);
  const int m = b - h, k1 = h - a;
  const size_t used = (size_t)m * k1;
  double *sp = work + used;
  const size_t sp_elems = work_elems > used ? work_elems - used : 0;
  // work = L(h:b, a:h) X(a:h, a:h)   (X11 lower)
  dgemm(s, 'N', 'N', m, k1, k1, 1.0, L + h + (size_t)a * ldl, ldl, X + a + (size_t)a * ldx, ldx, 0.0, work, m,
        kBLower, sp, sp_elems);
  // X(h:b, a:h) = -X(h:b, h:b) work   (X22 lower)
  dgemm(s, 'N', 'N', m, k1, m, -1.0, X + h + (size_t)h * ldx, ldx, work, m, 0.0, X + h + (size_t)a * ldx, ldx,
        kALower, sp, sp_elems);
}

void trtri_lower(cudaStream_t s, int n, const double *L, int ldl, double *X, int ldx, double *work,
                 size_t work_elems) {
  // X must start zero outside the blocks that are written.
  set_zero(s, X, (size_t)ldx * n);
  int nblk = ceil_div(n, NB);
  trtri_diag_kernel<<<nblk, 256, 0, s>>>(n, L, ldl, X, ldx);
  count_launch();
  trtri_rec(s, 0, n, L, ldl, X, ldx, work, work_elems);
}

// ------------------------------------------------------------------------------------- sytrd
// Blocked lower tridiagonalisation (LAPACK dsytrd/dlatrd semantics: panel of PB reflectors with the
// trailing-matrix update deferred to two rank-PB GEMMs per panel), Householder vectors explicit in V.
//
// All column steps of one panel run inside ONE cooperative (co-resident) kernel launch: the steps
// of a column are separated by a grid barrier instead of a kernel boundary, so a panel costs one
// launch and 4 barriers per column instead of 7 launches per column. Every reduction across CTAs
// goes through per-CTA partials summed in a fixed order, so results are deterministic.
constexpr int PB = 32;
constexpr int ST = 64;                 // symv tile
constexpr int kMaxPanelCtas = 4096;    // partial-sum slots per reduction
template <typename T>
struct PanelArgs {
  T *A;
  int lda, n, p0, nbp, ldv;
  T *Vp, *Wp, *y, *P, *dots, *part, *wpart, *dpart;
  T *V, *d, *e, *tau;
  GridBar *bar;
  unsigned epoch0;   // barriers completed by earlier panels of this reduction
  int *status;
};

// Sum of the G per-CTA partials p[0..G) in a fixed order (lane-strided, then a fixed shuffle tree);
// every CTA gets the same value. Called by all threads; result valid in all threads.
template <typename T>
__device__ T sum_partials(const T *p, int G, T *sh) {
  if (threadIdx.x < 32) {
    T s = T(0);
    for (int i = threadIdx.x; i < G; i += 32) s += __ldcg(p + i);
    s = warp_sum(s);
    if (threadIdx.x == 0) sh[0] = s;
  }
  __syncthreads();
  T r = sh[0];
  __syncthreads();
  return r;
}

// Decode a lower-triangle tile index into (row tile r, column tile c), c <= r.
__device__ __forceinline__ void tile_rc(int idx, int &r, int &c) {
  // single-precision estimate (FP64 is a slow pipe here), made exact by the integer corrections
  r = (int)((sqrtf(8.f * (float)idx + 1.f) - 1.f) * 0.5f);
  while ((r + 1) * (r + 2) / 2 <= idx) ++r;
  while (r * (r + 1) / 2 > idx) --r;
  c = idx - r * (r + 1) / 2;
}

// Element v(r) of the current reflector (absolute row r) from the updated column j: 0 above the
// subdiagonal, 1 on it, A(r, j) * scale below (every CTA forms it from the same data).
template <typename T>
__device__ __forceinline__ T reflector_elem(const T *colj, int j, int r, T scale) {
  return (r <= j) ? T(0) : ((r == j + 1) ? T(1) : __ldcg(colj + r) * scale);
}

// One panel of the reduction (columns p0 .. p0+nbp-1). Per column j (index jj in the panel):
//   A: finish W(:, jj-1) = w_raw + alpha v; A(j:n, j) -= V(j:n, 0:jj) W(j, 0:jj)^T + W V(j, :)^T;
//      partial sums of squares of A(j+2:n, j)
//   B: reflector (dlarfg: beta = -sign(alpha) ||x||, tau = (beta - alpha) / beta) formed by every
//      CTA from the partial sums; v stored; y = A22 v from 64x64 lower tiles of A22 = A(j+1:n, j+1:n)
//      (tiles double-buffered through registers) with v read from column j on the fly; dots
//      W(:,q)^T v and V(:,q)^T v
//   C: w_raw = tau (y - V (W^T v) - W (V^T v)) (kept in y), partial sums of w_raw^T v
// with alpha = -tau/2 w_raw^T v applied in the next A step (or after the last column). Three grid
// barriers per column. Rows are handled by 8 lanes each (the q sums and the tile-column sum of y
// split over the lanes, combined by a fixed shuffle tree).
template <typename T>
__global__ void __launch_bounds__(256) sytrd_panel_kernel(PanelArgs<T> a) {
  __shared__ T tile[ST][ST + 1];
  __shared__ T vr[ST], vc[ST];
  __shared__ T sh[32];
  __shared__ T cW[PB], cV[PB];
  __shared__ T s_scal[4];
  const int n = a.n, G = gridDim.x, b = blockIdx.x, t = threadIdx.x;
  const int lane8 = t & 7, grp = (t >> 3) & 3;
  const int wrow0 = (b * 256 + (t & ~31)) >> 3;    // 4 rows per warp, 8 lanes per row
  const int rstride = (G * 256) >> 3;
  const unsigned nb = (unsigned)G;
  unsigned epoch = a.epoch0;
  T alpha_prev = T(0);
  T *red = &tile[0][0];   // phase-A scratch (the tile is only used in phase B)
  for (int jj = 0; jj < a.nbp; ++jj) {
    const int j = a.p0 + jj;
    T *colj = a.A + (size_t)j * a.lda;
    // ------------------------------------------------------------------ A
    if (jj > 0) alpha_prev = T(-0.5) * __ldcg(a.tau + j - 1) * sum_partials(a.wpart, G, sh);
    const T *vprev = a.Vp + (size_t)(jj - 1) * n;
    if (t < jj) {
      T w = __ldcg(a.Wp + j + (size_t)t * n);
      if (t == jj - 1) w = __ldcg(a.y + j) + alpha_prev * __ldcg(vprev + j);
      cW[t] = w;
      cV[t] = __ldcg(a.Vp + j + (size_t)t * n);
    }
    __syncthreads();
    T sig = T(0);
    T pdv[4] = {T(0), T(0), T(0), T(0)}, pdw[4] = {T(0), T(0), T(0), T(0)};   // V/W(r, q) A(r, j), r >= j+2
    for (int rb = wrow0; rb < n; rb += rstride) {   // warp-uniform trip count (shuffles below)
      const int r = rb + grp;
      const bool in = r < n, act = in && r >= j;
      // issue every load of the row first
      T yv = T(0), vp = T(0), cj = T(0), vq[4], wv[4];
      if (jj > 0 && in) {
        yv = __ldcg(a.y + r);
        vp = __ldcg(vprev + r);
      }
      if (act) cj = __ldcg(colj + r);
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int q = lane8 + 8 * i;
        const bool use = act && q < jj;
        vq[i] = use ? __ldcg(a.Vp + r + (size_t)q * n) : T(0);
        wv[i] = (use && q != jj - 1) ? __ldcg(a.Wp + r + (size_t)q * n) : T(0);
      }
      const T wq = yv + alpha_prev * vp;
      if (jj > 0 && in && lane8 == 0) a.Wp[r + (size_t)(jj - 1) * n] = wq;
      T acc = T(0);
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int q = lane8 + 8 * i;
        if (act && q < jj) {
          acc = fma(vq[i], cW[q], acc);
          acc = fma((q == jj - 1) ? wq : wv[i], cV[q], acc);
        }
      }
      acc += __shfl_xor_sync(0xffffffffu, acc, 4);
      acc += __shfl_xor_sync(0xffffffffu, acc, 2);
      acc += __shfl_xor_sync(0xffffffffu, acc, 1);
      const T ar = cj - acc;   // updated A(r, j), identical in the 8 lanes
      if (act && lane8 == 0) {
        colj[r] = ar;
        if (r >= j + 2) sig = fma(ar, ar, sig);
      }
      if (act && r >= j + 2) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          pdv[i] = fma(vq[i], ar, pdv[i]);
          pdw[i] = fma((lane8 + 8 * i == jj - 1) ? wq : wv[i], ar, pdw[i]);
        }
      }
    }
    // per-CTA partials of the dots (fixed-order sum over the CTA's 32 row groups)
    if (jj > 0) {
      const int g32 = t >> 3;   // row group 0..31 of this CTA
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        red[g32 * 2 * PB + lane8 + 8 * i] = pdw[i];
        red[g32 * 2 * PB + PB + lane8 + 8 * i] = pdv[i];
      }
      __syncthreads();
      if (t < 2 * PB) {
        T sacc = T(0);
        for (int g2 = 0; g2 < 32; ++g2) sacc += red[g2 * 2 * PB + t];
        a.dpart[(size_t)b * 2 * PB + t] = sacc;
      }
    }
    sig = block_sum<256>(sig, sh);
    if (t == 0) a.part[b] = sig;
    grid_sync(a.bar, nb, epoch);
    // ------------------------------------------------------------------ B
    const int m = n - j - 1;
    const int nt = (m + ST - 1) / ST;
    {
      const T ss = sum_partials(a.part, G, sh);
      if (t == 0) {
        const T alpha = __ldcg(colj + j + 1);
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
        s_scal[0] = scale;
        if (b == 0) {
          a.d[j] = __ldcg(colj + j);
          a.e[j] = beta;
          a.tau[j] = tv;
        }
      }
      __syncthreads();
      const T scale = s_scal[0];
      for (int r = b * 256 + t; r < n; r += G * 256) {
        const T v = reflector_elem(colj, j, r, scale);
        a.Vp[r + (size_t)jj * n] = v;
        a.V[r + (size_t)j * a.ldv] = v;
      }
      // y = A22 v, tile by tile; the next tile's elements are loaded while this one is reduced
      const int ntiles = nt * (nt + 1) / 2;
      const T *A22 = a.A + (j + 1) + (size_t)(j + 1) * a.lda;
      const int ii = t & (ST - 1), jc = t >> 6;   // element (ii, jc + 4 q) of a tile, q < 16
      T reg[16], rv = T(0), cvv = T(0);
      int r = 0, c = 0;
      auto load_tile = [&](int idx) {
        tile_rc(idx, r, c);
        const int gi = r * ST + ii;
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int jt = jc + 4 * q, gj = c * ST + jt;
          reg[q] = (gi < m && gj < m && !(r == c && ii < jt)) ? A22[gi + (size_t)gj * a.lda] : T(0);
        }
        if (t < ST) {
          rv = (r * ST + t < m) ? reflector_elem(colj, j, j + 1 + r * ST + t, scale) : T(0);
          cvv = (c * ST + t < m) ? reflector_elem(colj, j, j + 1 + c * ST + t, scale) : T(0);
        }
      };
      int idx = b;
      if (idx < ntiles) load_tile(idx);
      // dots W(:,q)^T v and V(:,q)^T v = scale * sum_{r >= j+2} X(r, q) A(r, j) + X(j+1, q)
      for (int dq = b; dq < 2 * jj; dq += G) {
        const int q = dq % jj;
        const bool isV = dq >= jj;
        T s2 = T(0);
        for (int b2 = t; b2 < G; b2 += 256) s2 += __ldcg(a.dpart + (size_t)b2 * 2 * PB + (isV ? PB : 0) + q);
        s2 = block_sum<256>(s2, sh);
        if (t == 0) {
          const T x1 = __ldcg((isV ? a.Vp : a.Wp) + (j + 1) + (size_t)q * n);
          a.dots[(isV ? PB : 0) + q] = scale * s2 + x1;
        }
      }
      while (idx < ntiles) {
        const int tr = r, tc = c;
#pragma unroll
        for (int q = 0; q < 16; ++q) tile[ii][jc + 4 * q] = reg[q];
        if (t < ST) {
          vr[t] = rv;
          vc[t] = cvv;
        }
        __syncthreads();
        const int nidx = idx + G;
        if (nidx < ntiles) load_tile(nidx);
        if (tr == tc) {
          for (int k = t; k < ST * ST; k += 256) {
            const int i2 = k % ST, j2 = k / ST;
            if (i2 < j2) tile[i2][j2] = tile[j2][i2];
          }
          __syncthreads();
        }
        {
          const int row = t >> 2, part = t & 3;
          T s = T(0);
#pragma unroll
          for (int q = 0; q < 16; ++q) s = fma(tile[row][part * 16 + q], vc[part * 16 + q], s);
          s += __shfl_xor_sync(0xffffffffu, s, 1);
          s += __shfl_xor_sync(0xffffffffu, s, 2);
          if (part == 0) a.P[((size_t)tr * nt + tc) * ST + row] = s;
        }
        if (tc < tr) {
          const int colq = t >> 2, part = t & 3;
          T s = T(0);
#pragma unroll
          for (int q = 0; q < 16; ++q) s = fma(tile[part * 16 + q][colq], vr[part * 16 + q], s);
          s += __shfl_xor_sync(0xffffffffu, s, 1);
          s += __shfl_xor_sync(0xffffffffu, s, 2);
          if (part == 0) a.P[((size_t)tc * nt + tr) * ST + colq] = s;
        }
        __syncthreads();
        idx = nidx;
      }
    }
    grid_sync(a.bar, nb, epoch);
    // ------------------------------------------------------------------ C
    {
      if (t < jj) {
        cW[t] = __ldcg(a.dots + t);        // W(:,q)^T v
        cV[t] = __ldcg(a.dots + PB + t);   // V(:,q)^T v
      }
      __syncthreads();
      const T tv = __ldcg(a.tau + j);
      const T *v = a.Vp + (size_t)jj * n;
      T s = T(0);
      for (int rb = wrow0; rb < n; rb += rstride) {   // warp-uniform trip count
        const int r = rb + grp;
        const bool act = r > j && r < n;
        T acc = T(0), vrow = T(0), vq[4], wv[4];
        if (act) {
          vrow = __ldcg(v + r);
          const int rr = r - j - 1;
          const T *Pr = a.P + (size_t)(rr / ST) * nt * ST + (rr % ST);
#pragma unroll 4
          for (int c2 = lane8; c2 < nt; c2 += 8) acc += __ldcg(Pr + (size_t)c2 * ST);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int q = lane8 + 8 * i;
          const bool use = act && q < jj;
          vq[i] = use ? __ldcg(a.Vp + r + (size_t)q * n) : T(0);
          wv[i] = use ? __ldcg(a.Wp + r + (size_t)q * n) : T(0);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int q = lane8 + 8 * i;
          if (act && q < jj) {
            acc = fma(-vq[i], cW[q], acc);
            acc = fma(-wv[i], cV[q], acc);
          }
        }
        acc += __shfl_xor_sync(0xffffffffu, acc, 4);
        acc += __shfl_xor_sync(0xffffffffu, acc, 2);
        acc += __shfl_xor_sync(0xffffffffu, acc, 1);
        if (lane8 == 0 && r < n) {
          const T val = act ? tv * acc : T(0);
          a.y[r] = val;
          s = fma(val, vrow, s);
        }
      }
      s = block_sum<256>(s, sh);
      if (t == 0) a.wpart[b] = s;
    }
    grid_sync(a.bar, nb, epoch);
  }
  // finish the last column's W
  {
    const int jl = a.p0 + a.nbp - 1;
    const T al = T(-0.5) * __ldcg(a.tau + jl) * sum_partials(a.wpart, G, sh);
    const T *vl = a.Vp + (size_t)(a.nbp - 1) * n;
    for (int r = b * 256 + t; r < n; r += G * 256)
      a.Wp[r + (size_t)(a.nbp - 1) * n] = __ldcg(a.y + r) + al * __ldcg(vl + r);
  }
  if (t == 0 && a.status != nullptr && *(volatile int *)&a.bar->err != 0)
    atomicMax(a.status, (int)kDevIterCap);
}

template <typename T>
__global__ void copy_last_diag_kernel(int n, const T *A, int lda, T *d) {
  d[n - 1] = A[(n - 1) + (size_t)(n - 1) * lda];
}

template <typename T>
size_t sytrd_work_size(int n) {
  size_t nt = (size_t)ceil_div(n, ST);
  // Vp, Wp, a copy of Vp, y, P, dots, part, wpart, dpart, barrier (16 elements)
  return 3 * (size_t)n * PB + (size_t)n + nt * nt * ST + 2 * PB + 2 * (size_t)kMaxPanelCtas +
         2 * (size_t)PB * kMaxPanelCtas + 16;
}

// CTAs of the cooperative panel launch: every SM's resident share (at most 2 per SM).
template <typename T>
static int panel_ctas() {
  static int g = 0;
  if (g == 0) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sytrd_panel_kernel<T>, 256, 0);
    g = sms * std::max(1, std::min(per_sm, 2));
    g = std::min(g, kMaxPanelCtas);
  }
  return g;
}

template <typename T>
void sytrd_lower(cudaStream_t s, int n, T *A, int lda, T *d, T *e, T *tau, T *V, int ldv, T *work, int *status) {
  T *Vp = work;
  T *Wp = Vp + (size_t)n * PB;
  T *Vp2 = Wp + (size_t)n * PB;   // [Vp | Wp] and [Wp | Vp2] are n x 2 PB matrices
  T *y = Vp2 + (size_t)n * PB;
  T *P = y + n;
  size_t T0 = (size_t)ceil_div(n, ST);
  T *dots = P + T0 * T0 * ST;
  T *part = dots + 2 * PB;
  T *wpart = part + kMaxPanelCtas;
  T *dpart = wpart + kMaxPanelCtas;
  GridBar *bar = reinterpret_cast<GridBar *>(dpart + 2 * (size_t)PB * kMaxPanelCtas);
  set_zero_t<T>(s, V, (size_t)ldv * n);
  if (n == 1) {
    copy_last_diag_kernel<T><<<1, 1, 0, s>>>(n, A, lda, d);
    count_launch();
    return;
  }
  cudaMemsetAsync(bar, 0, sizeof(GridBar), s);
  PanelResidentPlan plan;
  const bool resident = g_panel_mode.load() != 0 && panel_resident_plan<T>(n, A, lda, plan);
  const int G = resident ? plan.ctas : panel_ctas<T>();
  unsigned epoch0 = 0;
  for (int p0 = 0; p0 < n - 1; p0 += PB) {
    int nbp = std::min(PB, n - 1 - p0);
    KernelTimer kt(s);
    if (resident) {
      // two grid barriers per column; wpart holds the per-CTA partials of v^T A22 v; epoch0 counts
      // barrier arrivals
      panel_resident_launch<T>(s, plan, plan.ctas, A, lda, n, p0, nbp, Vp, Wp, P, dots, part, wpart, dpart, V, ldv,
                               d, e, tau, bar, epoch0, status);
      epoch0 += 2u * (unsigned)nbp * (unsigned)plan.ctas;
    } else {
      PanelArgs<T> pa{A, lda, n, p0, nbp, ldv, Vp, Wp, y, P, dots, part, wpart, dpart, V, d, e, tau, bar, epoch0, status};
      epoch0 += 3u * (unsigned)nbp;
      void *args[] = {&pa};
      cudaLaunchCooperativeKernel((const void *)sytrd_panel_kernel<T>, dim3(G), dim3(256), args, 0, s);
      count_launch();
    }
    // algorithmic work per column j of the panel (m = n - j - 1): the FLOPs of the symmetric
    // matrix-vector product, 2 m^2 (the trailing rank-2k updates are counted with the GEMMs)
    double work = 0.0;
    for (int jj = 0; jj < nbp; ++jj) {
      const double m = (double)(n - (p0 + jj) - 1);
      work += 2.0 * m * m;
    }
    kt.done(sizeof(T) == 8 ? kPhKSytrdPanel : kPhKSytrdPanel32, work);
    int t0 = p0 + nbp;
    int m2 = n - t0;
    if (m2 > 0) {
      T *At = A + t0 + (size_t)t0 * lda;
      if (nbp == PB) {
        // one rank-2 PB update: A22 -= [V W] [W V]^T, with the copy of V placed after W
        cudaMemcpy2DAsync(Vp2 + t0, (size_t)n * sizeof(T), Vp + t0, (size_t)n * sizeof(T), (size_t)m2 * sizeof(T),
                          PB, cudaMemcpyDeviceToDevice, s);
        gemm<T>(s, 'N', 'T', m2, m2, 2 * PB, T(-1), Vp + t0, n, Wp + t0, n, T(1), At, lda, kCLower);
      } else {
        gemm<T>(s, 'N', 'T', m2, m2, nbp, T(-1), Vp + t0, n, Wp + t0, n, T(1), At, lda, kCLower);
        gemm<T>(s, 'N', 'T', m2, m2, nbp, T(-1), Wp + t0, n, Vp + t0, n, T(1), At, lda, kCLower);
      }
    }
  }
  copy_last_diag_kernel<T><<<1, 1, 0, s>>>(n, A, lda, d);
  count_launch();
}

// ------------------------------------------------------------------------------------- ormtr
constexpr int OB = 64;

// T (nb x nb, upper, nb <= OB) of the compact WY form: H_p..H_{p+nb-1} = I - V T V^T, from G = V^T V
// (leading dimension ldg), written to Tf (leading dimension ldt). The upper triangle of G is staged in
// shared memory first, so the serial recurrence T(0:i, i) = -tau_i T(0:i, 0:i) G(0:i, i) reads only
// shared memory.
template <typename T>
__global__ void larft_kernel(int nb, const T *G, int ldg, const T *tau, T *Tf, int ldt) {
  extern __shared__ __align__(16) unsigned char larft_smem[];
  T(*t)[OB + 1] = reinterpret_cast<T(*)[OB + 1]>(larft_smem);
  T(*g)[OB + 1] = t + OB;
  const int tid = threadIdx.x;
  for (int k = tid; k < OB * OB; k += blockDim.x) {
    const int r = k % OB, c = k / OB;
    t[r][c] = T(0);
    g[r][c] = (r <= c && c < nb) ? G[r + (size_t)c * ldg] : T(0);
  }
  __syncthreads();
  for (int i = 0; i < nb; ++i) {
    const T ti = tau[i];
    T v = T(0);
    if (tid < i) {
      for (int q = tid; q < i; ++q) v = fma(t[tid][q], g[q][i], v);
      v *= -ti;
    }
    __syncthreads();
    if (tid < i) t[tid][i] = v;
    if (tid == 0) t[i][i] = ti;
    __syncthreads();
  }
  for (int k = tid; k < nb * nb; k += blockDim.x) Tf[k % nb + (size_t)(k / nb) * ldt] = t[k % nb][k / nb];
}

template <typename T>
static void larft_launch(cudaStream_t s, int nb, const T *G, int ldg, const T *tau, T *Tf, int ldt) {
  constexpr int kSmem = 2 * OB * (OB + 1) * (int)sizeof(T);
  ensure_dyn_smem((const void *)larft_kernel<T>, kSmem);
  larft_kernel<T><<<1, OB, kSmem, s>>>(nb, G, ldg, tau, Tf, ldt);
  count_launch();
}

template <typename T>
void larft(cudaStream_t s, int nb, const T *G, const T *tau, T *Tf) {
  larft_launch<T>(s, nb, G, nb, tau, Tf, nb);
}
template void larft<float>(cudaStream_t, int, const float *, const float *, float *);
template void larft<double>(cudaStream_t, int, const double *, const double *, double *);

// Z is updated by blocks of OB2 reflectors: two larft blocks of OB merged into one compact WY form,
// T = [[T1, -T1 (V1^T V2) T2], [0, T2]] (H1 H2 = I - [V1 V2] T [V1 V2]^T), so that the two large
// products of a block have 128 rows and a K of 128.
constexpr int OB2 = 2 * OB;

template <typename T>
size_t ormtr_work_size(int n, int k) {
  // G, T (OB2 x OB2), X (OB x OB), M, M2 (OB2 x k) + split-K partials (8 slices of OB2 x max(k, OB2))
  return 2 * (size_t)OB2 * OB2 + (size_t)OB * OB + 2 * (size_t)OB2 * std::max(k, 1) +
         8 * (size_t)OB2 * std::max(k, OB2);
}

template <typename T>
void ormtr_left(cudaStream_t s, int n, int k, const T *V, int ldv, const T *tau, T *Z, int ldz, T *work) {
  if (n <= 1 || k <= 0) return;
  T *G = work;
  T *Tf = G + OB2 * OB2;
  T *X = Tf + OB2 * OB2;
  T *M = X + OB * OB;
  T *M2 = M + (size_t)OB2 * k;
  T *SP = M2 + (size_t)OB2 * k;
  const size_t sp_elems = 8 * (size_t)OB2 * std::max(k, OB2);
  int nref = n - 1;  // reflectors j = 0 .. n-2
  int last = ((nref - 1) / OB2) * OB2;
  for (int p0 = last; p0 >= 0; p0 -= OB2) {
    const int nb = std::min(OB2, nref - p0);
    const int n1 = std::min(nb, OB), n2 = nb - n1;
    int r0 = p0 + 1;          // first nonzero row of the block's vectors
    int mr = n - r0;
    const T *Vb = V + r0 + (size_t)p0 * ldv;
    gemm<T>(s, 'T', 'N', nb, nb, mr, T(1), Vb, ldv, Vb, ldv, T(0), G, nb, 0, SP, sp_elems);
    set_zero_t<T>(s, Tf, (size_t)nb * nb);
    larft_launch<T>(s, n1, G, nb, tau + p0, Tf, nb);
    if (n2 > 0) {
      larft_launch<T>(s, n2, G + n1 + (size_t)n1 * nb, nb, tau + p0 + n1, Tf + n1 + (size_t)n1 * nb, nb);
      // T12 = -T1 G12 T2 with G12 = V1^T V2: X = G12 T2, then T12 = -T1 X (T1, T2 upper)
      gemm<T>(s, 'N', 'N', n1, n2, n2, T(1), G + (size_t)n1 * nb, nb, Tf + n1 + (size_t)n1 * nb, nb, T(0), X, n1,
              kBUpper);
      gemm<T>(s, 'N', 'N', n1, n2, n1, T(-1), Tf, nb, X, n1, T(0), Tf + (size_t)n1 * nb, nb, kAUpper);
    }
    gemm<T>(s, 'T', 'N', nb, k, mr, T(1), Vb, ldv, Z + r0, ldz, T(0), M, nb, 0, SP, sp_elems);
    gemm<T>(s, 'N', 'N', nb, k, nb, T(1), Tf, nb, M, nb, T(0), M2, nb, kAUpper);
    gemm<T>(s, 'N', 'N', mr, k, nb, T(-1), Vb, ldv, M2, nb, T(1), Z + r0, ldz);
  }
}

template size_t sytrd_work_size<double>(int);
template size_t sytrd_work_size<float>(int);
template void sytrd_lower<double>(cudaStream_t, int, double *, int, double *, double *, double *, double *, int,
                                  double *, int *);
template void sytrd_lower<float>(cudaStream_t, int, float *, int, float *, float *, float *, float *, int, float *,
                                 int *);
template size_t ormtr_work_size<double>(int, int);
template size_t ormtr_work_size<float>(int, int);
template void ormtr_left<double>(cudaStream_t, int, int, const double *, int, const double *, double *, int,
                                 double *);
template void ormtr_left<float>(cudaStream_t, int, int, const float *, int, const float *, float *, int, float *);

}  // namespace dg
