// FP32-class GEMM on the tcgen05 tensor cores (sm_103a): C = alpha op(A) op(B) + beta C for FP32
// operands, computed exactly on BF16 digit slices, for the FP32 eigensolves of the mixed form.
//
// Splitting. Row i of op(A) gets a power-of-two scale 2^EA_i > max_k |A_ik|; each element is rounded
// to the 24-bit integer Y = round(|A_ik| 2^(24 - EA_i)) and recoded into three signed 8-bit digits,
// A_ik = sign 2^(EA_i - 24) (a_0 2^16 + a_1 2^8 + a_2) with a_0 in [0, 256] and a_1, a_2 in
// [-128, 127], integers that BF16 holds exactly. Columns of op(B) are split the same way (EB_j).
// Rounding Y is the only approximation of the operands: at most 2^-25 of the row (column) maximum.
//
// Products. The digit products with s + t = g are summed into one tensor-memory accumulator per
// group g = 0, 1, 2 (six products; groups 3 and 4 lie 2^-24 below the leading one and are dropped).
// Over one K-block of 64 a group sum is an integer of magnitude below 64 (2^16 + 2^15 + 2^15) <
// 2^22.3, so the FP32 accumulation in tensor memory is exact whatever its order. After each K-block
// the three sums are read back (exact float -> int32 conversion) and added into one int64 per output
// element as 2^16 G_0 + 2^8 G_1 + G_2; the epilogue scales it by 2^(EA_i + EB_j - 32) in FP64 and
// rounds to FP32. Integer accumulation makes the result independent of the order of the K-blocks.
//
// Accuracy: the error of C_ij is below about K max_k|A_ik| max_k|B_kj| 2^-23 plus the final
// rounding, FP32-class; the accumulation itself is exact (no rounding bias over long K).
//
// Kernel: one 128 x 64 output tile per CTA (256 threads), two stages of 3 + 3 digit slabs (72 KB each)
// copied with cp.async into 128-byte-swizzled shared memory, so the next K-block's copies run under
// the current block's 24 MMAs and readback. Every wait is bounded; on a timeout the kernel records an
// error, lets the MMAs drain, skips the output and releases its TMEM.
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>

#include "linalg.cuh"
#include "scratch.cuh"
#include "tcgen05.cuh"

namespace dg {

constexpr int FG_S = 3;                                   // digits per element
constexpr int FG_BM = 128, FG_BN = 64, FG_BK = 64;
constexpr int FG_THREADS = 256;
constexpr int FG_ATILE = FG_BM * FG_BK * 2;               // 16 KB: one digit slab of the A tile
constexpr int FG_BTILE = FG_BN * FG_BK * 2;               // 8 KB
constexpr int FG_STAGE = FG_S * (FG_ATILE + FG_BTILE);    // 72 KB
constexpr int FG_SMEM = 2 * FG_STAGE + 1024 + 64;         // two stages, alignment slack, barrier/slot/flag
constexpr uint32_t FG_TMEM_COLS = 256;                    // 3 groups x 64 columns, rounded to a power of two
constexpr int FG_GROUP_M = 8;                             // row tiles per group of the tile order

// Scale exponent E of a row from the bit pattern of its largest magnitude (FP32): max < 2^E.
__device__ __forceinline__ int fg_row_exp(unsigned maxbits) {
  const int ex = (int)(maxbits >> 23);
  return (ex < 1 ? 1 : ex) - 126;
}

// Three signed 8-bit digits of x at scale 2^E: x ~ 2^(E-24) (d0 2^16 + d1 2^8 + d2).
__device__ __forceinline__ void fg_digits(float x, int E, int *d) {
  const unsigned bits = __float_as_uint(x);
  const unsigned ab = bits & 0x7FFFFFFFu;
  int ex = (int)(ab >> 23);
  unsigned mant = ab & 0x7FFFFFu;
  if (ex) mant |= 1u << 23;
  else ex = 1;
  // |x| = mant 2^(ex - 150); Y = round(|x| 2^(24 - E)) = round(mant 2^(ex - 126 - E)), ex - 126 - E <= 0
  const int sh = ex - 126 - E;
  unsigned Y = 0;
  if (mant != 0 && ex < 255) {
    if (sh >= 0) Y = mant;   // only the row maximum's binade, sh == 0
    else if (sh > -32) Y = (unsigned)(((unsigned long long)mant + (1ull << (-sh - 1))) >> (-sh));
  }
  int v = (int)(Y & 255u);
  v -= (v >= 128) ? 256 : 0;
  d[2] = v;
  Y = (Y - (unsigned)v) >> 8;
  v = (int)(Y & 255u);
  v -= (v >= 128) ? 256 : 0;
  d[1] = v;
  Y = (Y - (unsigned)v) >> 8;
  d[0] = (int)Y;
  if (bits >> 31) {
    d[0] = -d[0];
    d[1] = -d[1];
    d[2] = -d[2];
  }
}

// Packing: two passes over the operand (rows R, K columns; element (r, k) = src[r * rs + k * ks], zero
// where the mask marks a structural zero: 1 keeps k <= r, 2 keeps k >= r), each on a grid of blocks
// of 32 rows x kFgPackChunk columns, so that a square operand of a few thousand rows spreads over
// every SM. Pass 1 (fg_rowmax_kernel) combines each row's largest magnitude into rmax[r] (its bit
// pattern; rmax zeroed beforehand) with atomicMax; pass 2 (fg_pack_kernel) writes the three digit
// slabs P[s * slab + r * Kp + k] (BF16, K-major, zero-padded to Kp columns and to the block's rows).
// 32 x 32 tiles through shared memory keep both the reads and the writes coalesced.
constexpr int kFgPackChunk = 256;

__device__ __forceinline__ void fg_load_tile(float (&tile)[32][33], int R, int K, const float *src, long long rs,
                                             long long ks, int mask, int r0, int k0) {
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const bool k_contig = (ks == 1);
#pragma unroll
  for (int q = ty; q < 32; q += 8) {
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
}

__global__ void __launch_bounds__(256) fg_rowmax_kernel(int R, int K, const float *src, long long rs, long long ks,
                                                        int mask, unsigned *rmax) {
  __shared__ float tile[32][33];
  const int r0 = blockIdx.x * 32, kc0 = blockIdx.y * kFgPackChunk;
  const int kc1 = min(K, kc0 + kFgPackChunk);
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  unsigned mx[4] = {0u, 0u, 0u, 0u};
  for (int k0 = kc0; k0 < kc1; k0 += 32) {
    __syncthreads();
    fg_load_tile(tile, R, K, src, rs, ks, mask, r0, k0);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const unsigned b = __float_as_uint(tile[ty + 8 * i][tx]) & 0x7FFFFFFFu;
      mx[i] = b > mx[i] ? b : mx[i];
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    unsigned v = mx[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned w = __shfl_xor_sync(0xffffffffu, v, o);
      v = w > v ? w : v;
    }
    if (tx == 0 && v != 0u) atomicMax(&rmax[r0 + ty + 8 * i], v);
  }
}

__global__ void __launch_bounds__(256) fg_pack_kernel(int R, int K, const float *src, long long rs, long long ks,
                                                      int mask, int Kp, size_t slab, __nv_bfloat16 *P,
                                                      const unsigned *rmax) {
  __shared__ float tile[32][33];
  const int r0 = blockIdx.x * 32, kc0 = blockIdx.y * kFgPackChunk;
  const int kc1 = min(Kp, kc0 + kFgPackChunk);
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  int E[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) E[i] = fg_row_exp(rmax[r0 + ty + 8 * i]);
  for (int k0 = kc0; k0 < kc1; k0 += 32) {
    __syncthreads();
    fg_load_tile(tile, R, K, src, rs, ks, mask, r0, k0);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int q = ty + 8 * i;
      int d[FG_S];
      fg_digits(tile[q][tx], E[i], d);
      __nv_bfloat16 *dst = P + (size_t)(r0 + q) * Kp + k0 + tx;
#pragma unroll
      for (int s = 0; s < FG_S; ++s) dst[(size_t)s * slab] = __float2bfloat16_rn((float)d[s]);
    }
  }
}

// Instruction descriptor: D FP32, A and B BF16, both K-major, M = 128, N = 64.
__host__ __device__ constexpr uint32_t fg_idesc() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(FG_BN >> 3) << 17) | ((uint32_t)(FG_BM >> 4) << 24);
}

__device__ __forceinline__ void fg_cp_async16(uint32_t dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}

// Packed operands: PA = three digit slabs of op(A) rows (each Mp x Kp), PB = three slabs of op(B)^T
// rows (each Np x Kp); rmaxA / rmaxB the row maxima of the packing pass. With P != nullptr the CTA
// (tile, z) sums only the z-th run of kb_split K-blocks and stores its int64 accumulators at
// P[z Mp Np + row + col Mp] (split-K; fg_splitk_reduce adds them exactly and scales).
__global__ void __launch_bounds__(FG_THREADS, 1) fg_gemm_kernel(int m, int n, int Kp, int Mp, int Np,
                                                              const __nv_bfloat16 *PA, const __nv_bfloat16 *PB,
                                                              const unsigned *rmaxA, const unsigned *rmaxB,
                                                              float alpha, float beta, float *C, int ldc, int flags,
                                                              int *err, long long *P, int kb_split) {
  extern __shared__ __align__(1024) unsigned char fg_smem_raw[];
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  // output tiles in groups of FG_GROUP_M row tiles (all column tiles of a group before the next)
  const int ntm = gridDim.x, ntn = gridDim.y;
  const int bid = blockIdx.x + ntm * blockIdx.y;
  const int first_m = bid / (FG_GROUP_M * ntn) * FG_GROUP_M;
  const int gm = min(ntm - first_m, FG_GROUP_M);
  const int local = bid % (FG_GROUP_M * ntn);
  const int i0 = (first_m + local % gm) * FG_BM, j0 = (local / gm) * FG_BN;
  if ((flags & kCLower) && j0 > i0 + FG_BM - 1) return;   // tile above the diagonal, before any TMEM use
  // K-blocks that can hold non-zero products (triangular operands)
  int kbeg = 0, kend = Kp;
  if (flags & kALower) kend = min(kend, i0 + FG_BM);
  if (flags & kAUpper) kbeg = max(kbeg, i0);
  if (flags & kBLower) kbeg = max(kbeg, j0);
  if (flags & kBUpper) kend = min(kend, j0 + FG_BN);
  int kb0 = kbeg / FG_BK, kb1 = (kend + FG_BK - 1) / FG_BK;
  if (P != nullptr) {
    kb0 += blockIdx.z * kb_split;
    kb1 = min(kb1, kb0 + kb_split);
  }
  const int nkb = kb1 > kb0 ? kb1 - kb0 : 0;

  const uint32_t raw = smem_u32(fg_smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  unsigned char *sm = fg_smem_raw + (base - raw);
  uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + 2 * FG_STAGE);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + 2 * FG_STAGE + 8);
  volatile int *sfail = reinterpret_cast<volatile int *>(sm + 2 * FG_STAGE + 16);
  if (t == 0) {
    mbar_init(smem_u32(mbar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *sfail = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(FG_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;

  const size_t slabA = (size_t)Mp * Kp, slabB = (size_t)Np * Kp;
  // Each thread copies the 16-byte chunk (t & 7) of rows t/8 + 32 j of every slab: 3 A slabs x 4 rows
  // and 3 B slabs x 2 rows. Within a swizzle atom of 8 rows the chunk index is XORed with row & 7,
  // which is (t / 8) & 7 for all rows of the thread.
  const int trow = t >> 3, tch = t & 7;
  const uint32_t soff = trow * 128 + ((tch ^ (trow & 7)) << 4);
  const __nv_bfloat16 *ga = PA + (size_t)(i0 + trow) * Kp + tch * 8;
  const __nv_bfloat16 *gb = PB + (size_t)(j0 + trow) * Kp + tch * 8;
  const size_t row32 = (size_t)32 * Kp;
  auto prefetch = [&](int kb, int st) {
    const uint32_t sdst = base + st * FG_STAGE + soff;
    const __nv_bfloat16 *pa = ga + (size_t)kb * FG_BK, *pb = gb + (size_t)kb * FG_BK;
#pragma unroll
    for (int sl = 0; sl < FG_S; ++sl) {
#pragma unroll
      for (int j = 0; j < 4; ++j) fg_cp_async16(sdst + sl * FG_ATILE + j * 4096, pa + j * row32);
#pragma unroll
      for (int j = 0; j < 2; ++j) fg_cp_async16(sdst + FG_S * FG_ATILE + sl * FG_BTILE + j * 4096, pb + j * row32);
      pa += slabA;
      pb += slabB;
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };

  const int quad = warp & 3, half = warp >> 2;
  long long acc[32];
#pragma unroll
  for (int c = 0; c < 32; ++c) acc[c] = 0;
  int drain = -1;   // thread 0: parity of the MMA commit whose wait timed out
  if (nkb > 0) prefetch(kb0, 0);
  for (int it = 0; it < nkb; ++it) {
    // the other stage was read by the MMAs of block it - 1, which completed in the last iteration
    if (it + 1 < nkb) {
      prefetch(kb0 + it + 1, (it + 1) & 1);
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (t == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t sa = base + (it & 1) * FG_STAGE;
      const uint64_t da0 = tc_sdesc(sa), db0 = tc_sdesc(sa + FG_S * FG_ATILE);
#pragma unroll
      for (int g = 0; g < FG_S; ++g)
#pragma unroll
        for (int s = 0; s <= g; ++s)
#pragma unroll
          for (int kk = 0; kk < FG_BK / 16; ++kk)
            tc_mma(tmem + (uint32_t)(g * FG_BN), da0 + (uint64_t)((s * FG_ATILE + kk * 32) >> 4),
                   db0 + (uint64_t)(((g - s) * FG_BTILE + kk * 32) >> 4), fg_idesc(), (s | kk) != 0 ? 1u : 0u);
      tc_commit(smem_u32(mbar));
      if (!mbar_wait(smem_u32(mbar), (uint32_t)(it & 1))) {
        *sfail = 1;
        drain = it & 1;
      }
    }
    __syncthreads();
    if (*sfail) break;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tlane = tmem + ((uint32_t)(quad * 32) << 16);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      uint32_t v0[16], v1[16], v2[16];
      tc_ld16(tlane + (uint32_t)(0 * FG_BN + half * 32 + h * 16), v0);
      tc_ld16(tlane + (uint32_t)(1 * FG_BN + half * 32 + h * 16), v1);
      tc_wait_ld2x16(v0, v1);
      tc_ld16(tlane + (uint32_t)(2 * FG_BN + half * 32 + h * 16), v2);
      asm volatile("tcgen05.wait::ld.sync.aligned;"
                   : "+r"(v2[0]), "+r"(v2[1]), "+r"(v2[2]), "+r"(v2[3]), "+r"(v2[4]), "+r"(v2[5]), "+r"(v2[6]),
                     "+r"(v2[7]), "+r"(v2[8]), "+r"(v2[9]), "+r"(v2[10]), "+r"(v2[11]), "+r"(v2[12]), "+r"(v2[13]),
                     "+r"(v2[14]), "+r"(v2[15])
                   :
                   : "memory");
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const long long g0 = __float2int_rn(__uint_as_float(v0[c]));
        const long long g1 = __float2int_rn(__uint_as_float(v1[c]));
        const long long g2 = __float2int_rn(__uint_as_float(v2[c]));
        acc[h * 16 + c] += g0 * 65536 + g1 * 256 + g2;
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  __syncthreads();
  const bool failed = *sfail != 0;
  if (failed && t == 0 && drain >= 0) mbar_wait(smem_u32(mbar), (uint32_t)drain);   // let in-flight MMAs drain
  if (!failed && P != nullptr) {
    long long *Pz = P + (size_t)blockIdx.z * Mp * Np;
    const int row = i0 + quad * 32 + lane;
#pragma unroll
    for (int c = 0; c < 32; ++c) Pz[row + (size_t)(j0 + half * 32 + c) * Mp] = acc[c];
  } else if (!failed) {
    const int row = i0 + quad * 32 + lane;
    if (row < m) {
      const unsigned ma = rmaxA[row];
      const int ea = fg_row_exp(ma) - 32;
      const bool bad_a = (ma >> 23) >= 255u;
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        const int col = j0 + half * 32 + c;
        if (col < n && (!(flags & kCLower) || row >= col)) {
          const unsigned mb = rmaxB[col];
          double x = ldexp((double)acc[c], ea + fg_row_exp(mb)) * (double)alpha;
          float *cp = C + row + (size_t)col * ldc;
          if (beta != 0.f) x = fma((double)beta, (double)*cp, x);
          float y = (float)x;
          if (bad_a || (mb >> 23) >= 255u) y = __uint_as_float(0x7FC00000u);
          *cp = y;
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(FG_TMEM_COLS) : "memory");
  }
  if (t == 0 && failed) atomicExch(err, 1);
}

// C = alpha 2^(EA_i + EB_j - 32) sum_z P[z] + beta C over the elements a split-K product computed.
__global__ void fg_splitk_reduce(int m, int n, int Mp, int Np, int splits, const long long *__restrict__ P,
                                 const unsigned *rmaxA, const unsigned *rmaxB, float alpha, float beta, float *C,
                                 int ldc, int lowerC) {
  const size_t total = (size_t)m * n;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
    const int row = (int)(idx % m), col = (int)(idx / m);
    if (lowerC && row < col) continue;
    long long v = 0;
    for (int z = 0; z < splits; ++z) v += P[(size_t)z * Mp * Np + row + (size_t)col * Mp];
    const unsigned ma = rmaxA[row], mb = rmaxB[col];
    double x = ldexp((double)v, fg_row_exp(ma) + fg_row_exp(mb) - 32) * (double)alpha;
    float *cp = C + row + (size_t)col * ldc;
    if (beta != 0.f) x = fma((double)beta, (double)*cp, x);
    float y = (float)x;
    if ((ma >> 23) >= 255u || (mb >> 23) >= 255u) y = __uint_as_float(0x7FC00000u);
    *cp = y;
  }
}

// ------------------------------------------------------------------------------ host side
thread_local bool g_tc_fgemm = false;          // gemm<float> routes here while set (calling thread only)
std::atomic<bool> g_tc_fgemm_mixed{true};      // dftbgpu_set_fp32_digit_products
constexpr int kFgSMs = 148;   // CTAs in flight (one per SM; GB300 has 152, a few may be taken)
static thread_local ThreadScratch t_fg;
enum { kFgSlabs = 0, kFgRmax = 1, kFgPart = 2 };

static int fg_round_up(int x, int q) { return (x + q - 1) / q * q; }

static int fg_splits(int m, int n, int k) {
  const long long tiles = (long long)ceil_div(m, FG_BM) * ceil_div(n, FG_BN);
  const int nkb = ceil_div(std::max(k, 1), FG_BK);
  if (tiles >= kFgSMs || nkb < 8) return 1;
  long long sp = (kFgSMs + tiles - 1) / tiles;
  sp = std::min<long long>(sp, nkb / 4);
  sp = std::min<long long>(sp, 16);
  return (int)std::max<long long>(sp, 1);
}

int tc_fgemm(cudaStream_t s, char ta, char tb, int m, int n, int k, float alpha, const float *A, int lda,
             const float *B, int ldb, float beta, float *C, int ldc, int flags) {
  if (m <= 0 || n <= 0) return 0;
  const int Mp = fg_round_up(m, FG_BM), Np = fg_round_up(n, FG_BN), Kp = fg_round_up(std::max(k, 1), FG_BK);
  DeviceScratch &ds = t_fg.current();
  int rc = scratch_reserve(ds.buf[kFgSlabs], (size_t)FG_S * ((size_t)Mp + Np) * Kp * sizeof(__nv_bfloat16));
  if (rc == 0) rc = scratch_reserve(ds.buf[kFgRmax], ((size_t)Mp + Np) * sizeof(unsigned));
  if (rc == 0 && !ds.err) {
    rc = scratch_err(ds);
    if (rc == 0) rc = (int)cudaFuncSetAttribute(fg_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, FG_SMEM);
  }
  if (rc != 0) return rc;
  __nv_bfloat16 *PA = static_cast<__nv_bfloat16 *>(ds.buf[kFgSlabs].p), *PB = PA + (size_t)FG_S * Mp * Kp;
  unsigned *rA = static_cast<unsigned *>(ds.buf[kFgRmax].p), *rB = rA + Mp;
  const bool TA = (ta == 'T' || ta == 't'), TB = (tb == 'T' || tb == 't');
  // op(A)(r, k) and op(B)^T(j, k) as strided views; structural zeros from the triangular flags
  const long long ars = TA ? lda : 1, aks = TA ? 1 : lda;
  const long long brs = TB ? 1 : ldb, bks = TB ? ldb : 1;
  const int amask = (flags & kALower) ? 1 : ((flags & kAUpper) ? 2 : 0);
  const int bmask = (flags & kBLower) ? 2 : ((flags & kBUpper) ? 1 : 0);
  rc = (int)cudaMemsetAsync(rA, 0, ((size_t)Mp + Np) * sizeof(unsigned), s);
  if (rc != 0) return rc;
  const int kcm = std::max(1, ceil_div(k, kFgPackChunk)), kcp = ceil_div(Kp, kFgPackChunk);
  fg_rowmax_kernel<<<dim3(Mp / 32, kcm), 256, 0, s>>>(m, k, A, ars, aks, amask, rA);
  fg_rowmax_kernel<<<dim3(Np / 32, kcm), 256, 0, s>>>(n, k, B, brs, bks, bmask, rB);
  fg_pack_kernel<<<dim3(Mp / 32, kcp), 256, 0, s>>>(m, k, A, ars, aks, amask, Kp, (size_t)Mp * Kp, PA, rA);
  fg_pack_kernel<<<dim3(Np / 32, kcp), 256, 0, s>>>(n, k, B, brs, bks, bmask, Kp, (size_t)Np * Kp, PB, rB);
  const int splits = fg_splits(m, n, k);
  long long *Pp = nullptr;
  int kb_split = 0;
  if (splits > 1) {
    rc = scratch_reserve(ds.buf[kFgPart], (size_t)splits * Mp * Np * sizeof(long long));
    if (rc != 0) return rc;
    Pp = static_cast<long long *>(ds.buf[kFgPart].p);
    kb_split = ceil_div(Kp / FG_BK, splits);
  }
  fg_gemm_kernel<<<dim3(Mp / FG_BM, Np / FG_BN, splits), FG_THREADS, FG_SMEM, s>>>(
      m, n, Kp, Mp, Np, PA, PB, rA, rB, alpha, beta, C, ldc, flags, ds.err, Pp, kb_split);
  count_launch(5);
  if (Pp) {
    const int rb = (int)std::min<long long>(((long long)m * n + 255) / 256, 152 * 8);
    fg_splitk_reduce<<<rb, 256, 0, s>>>(m, n, Mp, Np, splits, Pp, rA, rB, alpha, beta, C, ldc,
                                        (flags & kCLower) ? 1 : 0);
    count_launch();
  }
  return (int)cudaGetLastError();
}

int tc_fgemm_error() { return scratch_take_err(t_fg.current()); }

}  // namespace dg
