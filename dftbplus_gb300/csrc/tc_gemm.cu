// Tensor-core GEMM for the reduced-precision steps (sm_103a, tcgen05 + TMEM): C = alpha op(A) op(B)
// + beta C for FP32 operands as split-BF16 compensated products. Each operand is split three ways,
// A = A0 + A1 + A2 with A0 = bf16(A), A1 = bf16(A - A0), A2 = bf16(A - A0 - A1) (24 significant bits,
// the FP32 mantissa), and the six leading products A0B0 + A0B1 + A1B0 + A0B2 + A2B0 + A1B1 are
// accumulated in FP32 in tensor memory (relative error ~2^-22; the three-term form A0B0 + A0B1 +
// A1B0 keeps only ~17 bits, which stalls the perturbative SCC iterations above 1e-7 e).
//
// Operands are first packed by a tiled pass into K-major BF16 slabs (three per operand), padded to whole
// tiles (128 rows, 64 K) with zeros, with the triangular structure flags applied as masks. The main
// kernel then streams 128 x 64 tiles of the four slabs into 128-byte-swizzled shared memory (two
// stages), one elected thread issues 24 tcgen05.mma (6 products x 4 K-steps of 16) per K-block and
// commits them to an mbarrier, and the epilogue reads the 128 x 128 FP32 tile from TMEM with
// tcgen05.ld. Every wait is bounded; on a timeout the kernel records an error and releases its TMEM.
#include <cuda_bf16.h>

#include <atomic>

#include "linalg.cuh"
#include "scratch.cuh"
#include "tcgen05.cuh"

namespace dg {

constexpr int TC_BM = 128, TC_BN = 128, TC_BK = 64;
constexpr int TC_THREADS = 128;
constexpr int TC_TILE_BYTES = TC_BM * TC_BK * 2;               // 16 KB per BF16 tile
constexpr int TC_SPLIT = 3;                                    // BF16 pieces per operand
constexpr int TC_STAGE_BYTES = 2 * TC_SPLIT * TC_TILE_BYTES;   // A0..A2, B0..B2
constexpr int TC_SMEM_BYTES = 2 * TC_STAGE_BYTES + 2048;       // two stages + alignment + barriers

// ------------------------------------------------------------------------------ packing
// Element (r, k) of the packed operand (rows R, K columns) = src[r * rs + k * ks], zero where the
// mask says the operand is structurally zero (mask 1: keep k <= r, mask 2: keep k >= r), written as
// three BF16 pieces at P0/P1/P2[r * Kp + k]. 32 x 32 tiles through shared memory, coalesced on both
// sides.
__global__ void tc_pack_kernel(int R, int K, const float *src, long long rs, long long ks, int mask, int Kp,
                               __nv_bfloat16 *P0, __nv_bfloat16 *P1, __nv_bfloat16 *P2) {
  __shared__ float tile[32][33];
  const int r0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8 threads
  const bool k_contig = (ks == 1);
  for (int q = ty; q < 32; q += 8) {
    // read: consecutive threads along the contiguous source dimension
    const int r = k_contig ? r0 + q : r0 + tx;
    const int k = k_contig ? k0 + tx : k0 + q;
    float v = 0.f;
    if (r < R && k < K) {
      const bool keep = (mask == 0) || (mask == 1 && k <= r) || (mask == 2 && k >= r);
      if (keep) v = src[(long long)r * rs + (long long)k * ks];
    }
    if (k_contig) tile[q][tx] = v;
    else tile[tx][q] = v;
  }
  __syncthreads();
  for (int q = ty; q < 32; q += 8) {
    const int r = r0 + q, k = k0 + tx;
    const float v = tile[q][tx];
    const __nv_bfloat16 b0 = __float2bfloat16_rn(v);
    const float r1 = v - __bfloat162float(b0);
    const __nv_bfloat16 b1 = __float2bfloat16_rn(r1);
    const __nv_bfloat16 b2 = __float2bfloat16_rn(r1 - __bfloat162float(b1));
    P0[(size_t)r * Kp + k] = b0;
    P1[(size_t)r * Kp + k] = b1;
    P2[(size_t)r * Kp + k] = b2;
  }
}

// ------------------------------------------------------------------------------ kernel
// Instruction descriptor: D FP32, A and B BF16, both K-major, M = 128, N = 128.
__host__ __device__ constexpr uint32_t tc_idesc() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TC_BN >> 3) << 17) | ((uint32_t)(TC_BM >> 4) << 24);
}

// One 128 x 128 tile of C per CTA (128 threads). Packed operands: PA = three slabs of op(A) rows
// (each Mp x Kp), PB = three slabs of op(B)^T rows (each Np x Kp), K-major BF16.
__global__ void __launch_bounds__(TC_THREADS, 1) tc_gemm_kernel(int m, int n, int Kp, int Mp, int Np,
                                                              const __nv_bfloat16 *PA, const __nv_bfloat16 *PB,
                                                              float alpha, float beta, float *C, int ldc, int lowerC,
                                                              int *err) {
  extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int i0 = blockIdx.x * TC_BM, j0 = blockIdx.y * TC_BN;
  if (lowerC && j0 > i0 + TC_BM - 1) return;   // whole tile above the diagonal (before any TMEM use)
  const uint32_t raw = smem_u32(tc_smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  unsigned char *sm = tc_smem_raw + (base - raw);
  uint64_t *mbars = reinterpret_cast<uint64_t *>(sm + 2 * TC_STAGE_BYTES);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + 2 * TC_STAGE_BYTES + 32);
  if (t == 0) {
    mbar_init(smem_u32(&mbars[0]), 1);
    mbar_init(smem_u32(&mbars[1]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"((uint32_t)TC_BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const int nk = Kp / TC_BK;
  bool ok = true;
  const __nv_bfloat16 *src[2 * TC_SPLIT];
#pragma unroll
  for (int q = 0; q < TC_SPLIT; ++q) {
    src[q] = PA + (size_t)q * Mp * Kp + (size_t)i0 * Kp;
    src[TC_SPLIT + q] = PB + (size_t)q * Np * Kp + (size_t)j0 * Kp;
  }
  for (int kb = 0; kb < nk; ++kb) {
    const int s = kb & 1;
    unsigned char *stg = sm + s * TC_STAGE_BYTES;
    if (kb >= 2) {
      // the MMAs issued two K-blocks ago read this stage
      if (t == 0 && ok) ok = mbar_wait(smem_u32(&mbars[s]), ((kb - 2) >> 1) & 1);
      __syncthreads();
    }
#pragma unroll
    for (int mat = 0; mat < 2 * TC_SPLIT; ++mat) {
      const __nv_bfloat16 *g = src[mat] + kb * TC_BK;
      unsigned char *dst = stg + mat * TC_TILE_BYTES;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int chunk = t + q * TC_THREADS;   // 1024 chunks of 16 bytes per tile
        const int r = chunk >> 3, c = chunk & 7;
        const uint4 v = *reinterpret_cast<const uint4 *>(g + (size_t)r * Kp + c * 8);
        *reinterpret_cast<uint4 *>(dst + r * 128 + ((c ^ (r & 7)) << 4)) = v;
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (t == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t s0 = smem_u32(stg);
      // products A0B0, A0B1, A1B0, A0B2, A2B0, A1B1 (largest first)
      const int pa[6] = {0, 0, 1, 0, 2, 1}, pb[6] = {0, 1, 0, 2, 0, 1};
#pragma unroll
      for (int p = 0; p < 6; ++p)
#pragma unroll
        for (int kk = 0; kk < TC_BK / 16; ++kk)
          tc_mma(tmem, tc_sdesc(s0 + pa[p] * TC_TILE_BYTES + kk * 32),
                 tc_sdesc(s0 + (TC_SPLIT + pb[p]) * TC_TILE_BYTES + kk * 32), tc_idesc(),
                 (kb | p | kk) != 0 ? 1u : 0u);
      tc_commit(smem_u32(&mbars[s]));
    }
  }
  if (t == 0 && ok) ok = mbar_wait(smem_u32(&mbars[(nk - 1) & 1]), ((nk - 1) >> 1) & 1);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const int row = i0 + warp * 32 + lane;
#pragma unroll 1
  for (int cc = 0; cc < TC_BN / 32; ++cc) {
    uint32_t v[32];
    tc_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cc * 32), v);
#pragma unroll
    for (int q = 0; q < 32; ++q) {
      const int col = j0 + cc * 32 + q;
      if (row < m && col < n && (!lowerC || row >= col)) {
        float x = alpha * __uint_as_float(v[q]);
        if (beta != 0.f) x = fmaf(beta, C[row + (size_t)col * ldc], x);
        C[row + (size_t)col * ldc] = x;
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)TC_BN) : "memory");
  }
  if (t == 0 && !ok) atomicExch(err, 1);
}

// ------------------------------------------------------------------------------ host side
std::atomic<bool> g_tc_gemm{true};   // perturbative updates on the tensor cores (dftbgpu_set_tensor_cores)
static thread_local ThreadScratch t_tc;   // packed slabs of this thread on the current device

static int round_up(int x, int q) { return (x + q - 1) / q * q; }

int tc_gemm(cudaStream_t s, char ta, char tb, int m, int n, int k, float alpha, const float *A, int lda,
            const float *B, int ldb, float beta, float *C, int ldc, int flags) {
  if (m <= 0 || n <= 0) return 0;
  const int Mp = round_up(m, TC_BM), Np = round_up(n, TC_BN), Kp = round_up(std::max(k, 1), TC_BK);
  const size_t need = (size_t)TC_SPLIT * ((size_t)Mp + (size_t)Np) * Kp;
  DeviceScratch &ds = t_tc.current();
  int rc = scratch_reserve(ds.buf[0], need * sizeof(__nv_bfloat16));
  if (rc != 0) return rc;
  if (!ds.err) {
    rc = scratch_err(ds);
    if (rc == 0) rc = (int)cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM_BYTES);
    if (rc != 0) return rc;
  }
  __nv_bfloat16 *PA = static_cast<__nv_bfloat16 *>(ds.buf[0].p), *PB = PA + (size_t)TC_SPLIT * Mp * Kp;
  // op(A)(r, k) and op(B)^T(j, k) as strided views; structural zeros from the triangular flags
  const long long ars = (ta == 'N') ? 1 : lda, aks = (ta == 'N') ? lda : 1;
  const long long brs = (tb == 'N') ? ldb : 1, bks = (tb == 'N') ? 1 : ldb;
  const int amask = (flags & kALower) ? 1 : ((flags & kAUpper) ? 2 : 0);
  const int bmask = (flags & kBLower) ? 2 : ((flags & kBUpper) ? 1 : 0);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(s, &cap);
  const bool prof = g_gemm_prof.on && cap == cudaStreamCaptureStatusNone;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (prof) {
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
  }
  const size_t sa = (size_t)Mp * Kp, sb = (size_t)Np * Kp;
  tc_pack_kernel<<<dim3(Kp / 32, Mp / 32), 256, 0, s>>>(m, k, A, ars, aks, amask, Kp, PA, PA + sa, PA + 2 * sa);
  tc_pack_kernel<<<dim3(Kp / 32, Np / 32), 256, 0, s>>>(n, k, B, brs, bks, bmask, Kp, PB, PB + sb, PB + 2 * sb);
  tc_gemm_kernel<<<dim3(Mp / TC_BM, Np / TC_BN), TC_THREADS, TC_SMEM_BYTES, s>>>(
      m, n, Kp, Mp, Np, PA, PB, alpha, beta, C, ldc, (flags & kCLower) ? 1 : 0, ds.err);
  count_launch(3);
  if (prof) {
    cudaEventRecord(e1, s);
    g_gemm_prof.ev.push_back(e0);
    g_gemm_prof.ev.push_back(e1);
    g_gemm_prof.flops.push_back(((flags & kCLower) ? 1.0 : 2.0) * m * (double)n * k);
    g_gemm_prof.phase.push_back(kPhGemm32);
  }
  return (int)cudaGetLastError();
}

int tc_gemm_error() { return scratch_take_err(t_tc.current()); }

}  // namespace dg
