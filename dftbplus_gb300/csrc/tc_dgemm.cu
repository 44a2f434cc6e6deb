// FP64-class GEMM on the tcgen05 tensor cores (sm_103a): C = alpha op(A) op(B) + beta C for FP64
// operands, computed exactly on BF16 digit slices (an Ozaki-type splitting). GB300 issues FP64 FMAs
// at about 2 per clock per SM, its BF16 tensor cores about 4,000 multiply-adds per clock per SM, so
// 36 exact BF16 digit products still run well ahead of FP64 arithmetic.
//
// Splitting. Row i of op(A) gets a power-of-two scale 2^EA_i > max_k |A_ik|. Each element is
// rounded to the 55-bit fixed-point integer Y = round(|A_ik| 2^(55 - EA_i)) and recoded into eight
// signed 7-bit digits, A_ik = sign 2^(EA_i - 55) sum_s a_s 2^(7 (7 - s)) with a_0 in [0, 64] and
// a_s in [-64, 63] for s >= 1, so every digit is an integer that BF16 holds exactly. Columns of
// op(B) are split the same way (EB_j). Rounding Y is the only approximation of the operands: at most
// 2^-56 of the row (column) maximum.
//
// Products. The digit products with s + t = g are summed into one tensor-memory accumulator per
// group g = 0..7 (36 products; the groups g >= 8 lie 2^-56 below the leading one and are dropped).
// Over one K-block of 64 each group sum is an integer of magnitude <= 8 * 64 * 2^12 = 2^21, so the
// FP32 accumulation in tensor memory is exact whatever its rounding. After each K-block the eight
// sums are read back, converted to int32 exactly (adding 1.5 * 2^23 leaves an integer |v| <= 2^22 in
// the low mantissa bits), combined in pairs 2^7 G_g + G_{g+1} (int32) and added into one int64
// fixed-point accumulator per output element with weights 2^(7 (7 - g) - R); R = ceil(log2 Kp) - 1
// keeps the int64 clear of overflow (the weights of groups 6 and 7 become rounding right shifts: at
// most half a unit of 2^(EA_i + EB_j - 61 + R) per K-block and group). The epilogue scales the int64
// by 2^(EA_i + EB_j - 61 + R) in FP64. Integer accumulation makes the result independent of the
// order of the K-blocks.
//
// Accuracy: the error of C_ij is below K max_k|A_ik| max_k|B_kj| (2^-53 + K 2^-65), FP64-class
// (a native FP64 GEMM's bound is K 2^-53 sum_k |A_ik| |B_kj|); a row or column of op(A), op(B) that
// holds Inf or NaN gives NaN outputs.
//
// Kernel: one 128 x 64 output tile per CTA (256 threads). Per K-block the 8 + 8 digit slabs of the
// A and B tiles (192 KB) are copied with cp.async into 128-byte-swizzled shared memory, one thread
// issues the 144 tcgen05.mma (36 products x 4 K-steps of 16, M = 128, N = 64) into eight 64-column
// TMEM accumulators and commits them to an mbarrier; after the bounded wait the next K-block's copies
// are started and the eight warps read the group sums back (two warps per 32-lane TMEM quadrant, 32
// columns each). Every wait is bounded; on a timeout the kernel records an error, skips the output
// and releases its TMEM.
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <type_traits>

#include "linalg.cuh"
#include "scratch.cuh"
#include "tcgen05.cuh"
#include "tma.cuh"

namespace dg {

constexpr int DG_S = 8;                                   // digits per element
constexpr int DG_BM = 128, DG_BN = 64, DG_BK = 64;
constexpr int DG_THREADS = 256;
constexpr int DG_ATILE = DG_BM * DG_BK * 2;               // 16 KB: one digit slab of the A tile
constexpr int DG_BTILE = DG_BN * DG_BK * 2;               // 8 KB: one digit slab of the B tile
constexpr int DG_STAGE = DG_S * (DG_ATILE + DG_BTILE);    // 192 KB
constexpr int DG_SMEM = DG_STAGE + 1024 + 64;             // alignment slack + barrier, TMEM slot, flag
constexpr uint32_t DG_TMEM_COLS = 512;                    // 8 groups x 64 columns
constexpr int DG_GROUP_M = 8;                             // row tiles per group of the tile order

// Scale exponent E of a row from the bit pattern of its largest magnitude: max < 2^E.
__device__ __forceinline__ int dg_row_exp(unsigned long long maxbits) {
  const int ex = (int)(maxbits >> 52);
  return (ex < 1 ? 1 : ex) - 1022;
}

// Eight signed 7-bit digits of x at scale 2^E (see the header): x ~ 2^(E-55) sum_s d_s 2^(7(7-s)).
__device__ __forceinline__ void dg_digits(double x, int E, int *d) {
  const long long bits = __double_as_longlong(x);
  const unsigned long long ab = (unsigned long long)bits & 0x7FFFFFFFFFFFFFFFull;
  int ex = (int)(ab >> 52);
  unsigned long long mant = ab & 0xFFFFFFFFFFFFFull;
  if (ex) mant |= 1ull << 52;
  else ex = 1;
  // |x| = mant 2^(ex - 1075); Y = round(|x| 2^(55 - E)) = round(mant 2^(ex - 1020 - E)) < 2^55
  const int sh = ex - 1020 - E;
  unsigned long long Y = 0;
  if (mant != 0 && ex < 2047) {
    if (sh >= 0) Y = mant << (sh > 2 ? 2 : sh);   // sh <= 2 whenever |x| < 2^E
    else if (sh > -64) Y = (mant + (1ull << (-sh - 1))) >> (-sh);
  }
#pragma unroll
  for (int s = DG_S - 1; s >= 1; --s) {
    int v = (int)(Y & 127ull);
    v -= (v >= 64) ? 128 : 0;
    d[s] = v;
    Y = (Y - (unsigned long long)(long long)v) >> 7;
  }
  d[0] = (int)Y;
  if (bits < 0) {
#pragma unroll
    for (int s = 0; s < DG_S; ++s) d[s] = -d[s];
  }
}

// ------------------------------------------------------------------------------ packing
// Two passes over the operand (rows R, K columns; element (r, k) = src[r * rs + k * ks], zero where
// the mask marks a structural zero: 1 keeps k <= r, 2 keeps k >= r), each on a grid of blocks of 32
// rows x kDgPackChunk columns, so that a square operand of a few thousand rows spreads over every
// SM. Pass 1 (dg_rowmax_kernel) combines each row's largest magnitude into rmax[r] (its bit pattern,
// so that unsigned order is magnitude order; rmax zeroed beforehand) with atomicMax; pass 2
// (dg_pack_kernel) writes the eight digit slabs P[s * slab + r * Kp + k] (BF16, K-major, zero-padded
// to Kp columns and to the block's rows). 32 x 32 tiles through shared memory keep both the reads and
// the writes coalesced.
constexpr int kDgPackChunk = 256;

__device__ __forceinline__ void dg_load_tile(double (&tile)[32][33], int R, int K, const double *src, long long rs,
                                             long long ks, int mask, int r0, int k0) {
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const bool k_contig = (ks == 1);
#pragma unroll
  for (int q = ty; q < 32; q += 8) {
    const int r = k_contig ? r0 + q : r0 + tx;
    const int k = k_contig ? k0 + tx : k0 + q;
    double v = 0.0;
    if (r < R && k < K) {
      const bool keep = (mask == 0) || (mask == 1 && k <= r) || (mask == 2 && k >= r);
      if (keep) v = src[(long long)r * rs + (long long)k * ks];
    }
    if (k_contig) tile[q][tx] = v;
    else tile[tx][q] = v;
  }
}

__global__ void __launch_bounds__(256) dg_rowmax_kernel(int R, int K, const double *src, long long rs, long long ks,
                                                        int mask, unsigned long long *rmax) {
  __shared__ double tile[32][33];
  const int r0 = blockIdx.x * 32, kc0 = blockIdx.y * kDgPackChunk;
  const int kc1 = min(K, kc0 + kDgPackChunk);
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  unsigned long long mx[4] = {0ull, 0ull, 0ull, 0ull};
  for (int k0 = kc0; k0 < kc1; k0 += 32) {
    __syncthreads();
    dg_load_tile(tile, R, K, src, rs, ks, mask, r0, k0);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const unsigned long long b =
          (unsigned long long)__double_as_longlong(tile[ty + 8 * i][tx]) & 0x7FFFFFFFFFFFFFFFull;
      mx[i] = b > mx[i] ? b : mx[i];
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    unsigned long long v = mx[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
      v = w > v ? w : v;
    }
    if (tx == 0 && v != 0ull) atomicMax(&rmax[r0 + ty + 8 * i], v);
  }
}

__global__ void __launch_bounds__(256) dg_pack_kernel(int R, int K, const double *src, long long rs, long long ks,
                                                      int mask, int Kp, size_t slab, __nv_bfloat16 *P,
                                                      const unsigned long long *rmax) {
  __shared__ double tile[32][33];
  const int r0 = blockIdx.x * 32, kc0 = blockIdx.y * kDgPackChunk;
  const int kc1 = min(Kp, kc0 + kDgPackChunk);
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  int E[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) E[i] = dg_row_exp(rmax[r0 + ty + 8 * i]);
  for (int k0 = kc0; k0 < kc1; k0 += 32) {
    __syncthreads();
    dg_load_tile(tile, R, K, src, rs, ks, mask, r0, k0);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int q = ty + 8 * i;
      int d[DG_S];
      dg_digits(tile[q][tx], E[i], d);
      __nv_bfloat16 *dst = P + (size_t)(r0 + q) * Kp + k0 + tx;
#pragma unroll
      for (int s = 0; s < DG_S; ++s) dst[(size_t)s * slab] = __float2bfloat16_rn((float)d[s]);
    }
  }
}

// ------------------------------------------------------------------------------ kernel
// Instruction descriptor: D FP32, A and B BF16, both K-major, M = 128, N = 64.
__host__ __device__ constexpr uint32_t dg_idesc() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(DG_BN >> 3) << 17) | ((uint32_t)(DG_BM >> 4) << 24);
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}

// Packed operands: PA = eight digit slabs of op(A) rows (each Mp x Kp), PB = eight slabs of op(B)^T
// rows (each Np x Kp); rmaxA / rmaxB the row maxima of the packing pass. With P != nullptr the CTA
// (x, y, z) sums only the z-th run of kb_split K-blocks and stores its raw int64 accumulators at
// P[z Mp Np + row + col Mp] (split-K; dg_splitk_reduce adds them exactly and scales).
__global__ void __launch_bounds__(DG_THREADS, 1) dg_gemm_kernel(int m, int n, int Kp, int Mp, int Np,
                                                              const __nv_bfloat16 *PA, const __nv_bfloat16 *PB,
                                                              const unsigned long long *rmaxA,
                                                              const unsigned long long *rmaxB, int R, double alpha,
                                                              double beta, double *C, int ldc, int flags, int *err,
                                                              long long *P, int kb_split) {
  extern __shared__ __align__(1024) unsigned char dg_smem_raw[];
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  // output tiles in groups of DG_GROUP_M row tiles (all column tiles of a group before the next), so
  // that the CTAs resident at one time share the K-slices of a few A panels in L2
  const int ntm = gridDim.x, ntn = gridDim.y;
  const int bid = blockIdx.x + ntm * blockIdx.y;
  const int first_m = bid / (DG_GROUP_M * ntn) * DG_GROUP_M;
  const int gm = min(ntm - first_m, DG_GROUP_M);
  const int local = bid % (DG_GROUP_M * ntn);
  const int i0 = (first_m + local % gm) * DG_BM, j0 = (local / gm) * DG_BN;
  if ((flags & kCLower) && j0 > i0 + DG_BM - 1) return;   // tile above the diagonal, before any TMEM use
  // K-blocks that can hold non-zero products (triangular operands), as in the FP64 GEMM
  int kbeg = 0, kend = Kp;
  if (flags & kALower) kend = min(kend, i0 + DG_BM);
  if (flags & kAUpper) kbeg = max(kbeg, i0);
  if (flags & kBLower) kbeg = max(kbeg, j0);
  if (flags & kBUpper) kend = min(kend, j0 + DG_BN);
  int kb0 = kbeg / DG_BK, kb1 = (kend + DG_BK - 1) / DG_BK;
  if (P != nullptr) {
    kb0 += blockIdx.z * kb_split;
    kb1 = min(kb1, kb0 + kb_split);
  }
  const int nkb = kb1 > kb0 ? kb1 - kb0 : 0;

  const uint32_t raw = smem_u32(dg_smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  unsigned char *sm = dg_smem_raw + (base - raw);
  uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + DG_STAGE);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + DG_STAGE + 8);
  volatile int *sfail = reinterpret_cast<volatile int *>(sm + DG_STAGE + 16);
  if (t == 0) {
    mbar_init(smem_u32(mbar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *sfail = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(DG_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;

  const size_t slabA = (size_t)Mp * Kp, slabB = (size_t)Np * Kp;
  // Each thread copies the 16-byte chunk (t & 7) of rows t/8 + 32 j of every slab: 8 A slabs x 4 rows
  // and 8 B slabs x 2 rows, 48 copies. Within a swizzle atom of 8 rows the chunk index is XORed with
  // row & 7, which is (t / 8) & 7 for all rows of the thread.
  const int trow = t >> 3, tch = t & 7;
  const uint32_t sdst = base + trow * 128 + ((tch ^ (trow & 7)) << 4);
  const __nv_bfloat16 *ga = PA + (size_t)(i0 + trow) * Kp + tch * 8;
  const __nv_bfloat16 *gb = PB + (size_t)(j0 + trow) * Kp + tch * 8;
  const size_t row32 = (size_t)32 * Kp;
  auto prefetch = [&](int kb) {
    const __nv_bfloat16 *pa = ga + (size_t)kb * DG_BK, *pb = gb + (size_t)kb * DG_BK;
#pragma unroll
    for (int sl = 0; sl < DG_S; ++sl) {
#pragma unroll
      for (int j = 0; j < 4; ++j) cp_async16(sdst + sl * DG_ATILE + j * 4096, pa + j * row32);
#pragma unroll
      for (int j = 0; j < 2; ++j) cp_async16(sdst + DG_S * DG_ATILE + sl * DG_BTILE + j * 4096, pb + j * row32);
      pa += slabA;
      pb += slabB;
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };

  const int quad = warp & 3, half = warp >> 2;
  long long acc[32];
#pragma unroll
  for (int c = 0; c < 32; ++c) acc[c] = 0;
  if (nkb > 0) prefetch(kb0);
  for (int it = 0; it < nkb; ++it) {
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (t == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // descriptors of the stage's first A and B slabs; the others differ only in the start address
      // field (address / 16, no carry out of its 14 bits below 256 KB of shared memory)
      const uint64_t da0 = tc_sdesc(base), db0 = tc_sdesc(base + DG_S * DG_ATILE);
#pragma unroll
      for (int g = 0; g < DG_S; ++g)
#pragma unroll
        for (int s = 0; s <= g; ++s)
#pragma unroll
          for (int kk = 0; kk < DG_BK / 16; ++kk)
            tc_mma(tmem + (uint32_t)(g * DG_BN), da0 + (uint64_t)((s * DG_ATILE + kk * 32) >> 4),
                   db0 + (uint64_t)(((g - s) * DG_BTILE + kk * 32) >> 4), dg_idesc(), (s | kk) != 0 ? 1u : 0u);
      tc_commit(smem_u32(mbar));
      if (!mbar_wait(smem_u32(mbar), (uint32_t)(it & 1))) *sfail = 1;
    }
    __syncthreads();
    if (*sfail) break;
    if (it + 1 < nkb) prefetch(kb0 + it + 1);   // shared memory is free once the MMAs completed
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // groups in pairs (g, g + 1): p = 2^7 G_g + G_{g+1} fits int32 (|p| < 2^28.1) and enters the
    // int64 with the weight of g + 1; the magic-number offsets of both raw words cancel in one add
    const uint32_t tlane = tmem + ((uint32_t)(quad * 32) << 16);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
#pragma unroll
      for (int g = 0; g < DG_S; g += 2) {
        uint32_t va[16], vb[16];
        tc_ld16(tlane + (uint32_t)(g * DG_BN + half * 32 + h * 16), va);
        tc_ld16(tlane + (uint32_t)((g + 1) * DG_BN + half * 32 + h * 16), vb);
        tc_wait_ld2x16(va, vb);
        const int sh = 7 * (DG_S - 2 - g) - R;
#pragma unroll
        for (int c = 0; c < 16; ++c) {
          const uint32_t ba = (uint32_t)__float_as_int(__uint_as_float(va[c]) + 12582912.0f);
          const uint32_t bb = (uint32_t)__float_as_int(__uint_as_float(vb[c]) + 12582912.0f);
          const int p = (int)((ba << 7) + bb - 0x4B400000u * 129u);
          long long &a = acc[h * 16 + c];
          if (sh >= 0) a += (long long)p << sh;
          else a += (long long)((p + (1 << (-sh - 1))) >> (-sh));
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  __syncthreads();
  const bool failed = *sfail != 0;
  if (failed && t == 0) mbar_wait(smem_u32(mbar), (uint32_t)((nkb - 1) & 1));   // let in-flight MMAs drain
  if (!failed && P != nullptr) {
    long long *Pz = P + (size_t)blockIdx.z * Mp * Np;
    const int row = i0 + quad * 32 + lane;
#pragma unroll
    for (int c = 0; c < 32; ++c) Pz[row + (size_t)(j0 + half * 32 + c) * Mp] = acc[c];
  } else if (!failed) {
    const int row = i0 + quad * 32 + lane;
    if (row < m) {
      const unsigned long long ma = rmaxA[row];
      const int ea = dg_row_exp(ma) - 61 + R;
      const bool bad_a = (ma >> 52) >= 2047ull;
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        const int col = j0 + half * 32 + c;
        if (col < n && (!(flags & kCLower) || row >= col)) {
          const unsigned long long mb = rmaxB[col];
          double x = ldexp((double)acc[c], ea + dg_row_exp(mb));
          if (bad_a || (mb >> 52) >= 2047ull) x = __longlong_as_double(0x7FF8000000000000ll);
          x *= alpha;
          double *cp = C + row + (size_t)col * ldc;
          if (beta != 0.0) x = fma(beta, *cp, x);
          *cp = x;
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(DG_TMEM_COLS) : "memory");
  }
  if (t == 0 && failed) atomicExch(err, 1);
}

// ------------------------------------------------------------------------------ pipelined kernel
// The same products and exactness argument as dg_gemm_kernel, organised as a pipeline:
//   * one TMA load per operand and K-sub-block of 32 brings all eight digit slabs of the A (128 x 32)
//     and B (64 x 32) tiles into shared memory with the 64-byte swizzle (96 KB per stage, two
//     stages), from 3D tensor maps over the packed slabs (K, row, slab);
//   * thread 0 issues the 72 MMAs of a sub-block (36 products x 2 K-steps of 16) and commits them to
//     the stage's "empty" barrier; the load two sub-blocks ahead waits only for that barrier, so the
//     copies run under the MMAs;
//   * the eight group sums stay in TMEM for a window of 8 sub-blocks (K = 256): a group sum is an
//     integer of magnitude <= 8 x 256 x 2^12 = 2^23, still exact in FP32 whatever the order of the
//     additions; at the end of a window all eight warps read the sums back (an exact float -> int32
//     conversion; 2^7 G_g + G_{g+1} < 2^31) into the int64 accumulators, while the next window's
//     first copies are in flight;
//   * output tiles are visited in groups of 8 row tiles (all column tiles of a group before the next
//     group), so the CTAs resident at one time share the K-slices of 8 A panels and of the column
//     panels they walk, which stay in L2.
constexpr int DG2_SK = 32;                                  // K per sub-block (one stage)
constexpr int DG2_WIN = 8;                                  // sub-blocks per TMEM readback window
constexpr int DG2_ASLAB = DG_BM * DG2_SK * 2;               // 8 KB: one digit slab of the A tile
constexpr int DG2_BSLAB = DG_BN * DG2_SK * 2;               // 4 KB
constexpr int DG2_STAGE = DG_S * (DG2_ASLAB + DG2_BSLAB);   // 96 KB
constexpr int DG2_SMEM = 2 * DG2_STAGE + 1024 + 128;        // alignment slack + barriers, TMEM slot, flag

// Shared-memory matrix descriptor: K-major operand tile with the 64-byte swizzle (64-byte rows of 32
// BF16), 8-row groups 512 B apart.
__device__ __forceinline__ uint64_t dg2_sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);   // start address
  d |= (uint64_t)1 << 16;                     // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(512 >> 4) << 32;            // stride byte offset between 8-row groups
  d |= (uint64_t)1 << 46;                     // descriptor version
  d |= (uint64_t)4 << 61;                     // 64-byte swizzle
  return d;
}

__device__ __forceinline__ void dg2_arrive_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void dg2_tma3(uint32_t dst, const void *map, int x, int y, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          dst),
      "l"(map), "r"(x), "r"(y), "r"(0), "r"(mbar)
      : "memory");
}

__global__ void __launch_bounds__(DG_THREADS, 1) dg_gemm_tma_kernel(
    const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, int m, int n, int Kp,
    int Mp, int Np, const unsigned long long *rmaxA, const unsigned long long *rmaxB, int R, double alpha,
    double beta, double *C, int ldc, int flags, int *err, long long *P, int kb_split) {
  extern __shared__ __align__(1024) unsigned char dg_smem_raw[];
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  // grouped tile order
  const int ntm = gridDim.x, ntn = gridDim.y;
  const int bid = blockIdx.x + ntm * blockIdx.y;
  const int first_m = bid / (DG_GROUP_M * ntn) * DG_GROUP_M;
  const int gm = min(ntm - first_m, DG_GROUP_M);
  const int local = bid % (DG_GROUP_M * ntn);
  const int i0 = (first_m + local % gm) * DG_BM, j0 = (local / gm) * DG_BN;
  if ((flags & kCLower) && j0 > i0 + DG_BM - 1) return;   // tile above the diagonal, before any TMEM use
  int kbeg = 0, kend = Kp;
  if (flags & kALower) kend = min(kend, i0 + DG_BM);
  if (flags & kAUpper) kbeg = max(kbeg, i0);
  if (flags & kBLower) kbeg = max(kbeg, j0);
  if (flags & kBUpper) kend = min(kend, j0 + DG_BN);
  int kb0 = kbeg / DG_BK, kb1 = (kend + DG_BK - 1) / DG_BK;
  if (P != nullptr) {
    kb0 += blockIdx.z * kb_split;
    kb1 = min(kb1, kb0 + kb_split);
  }
  const int nsub = kb1 > kb0 ? 2 * (kb1 - kb0) : 0;
  const int kfirst = kb0 * DG_BK;

  const uint32_t raw = smem_u32(dg_smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  unsigned char *sm = dg_smem_raw + (base - raw);
  uint64_t *bars = reinterpret_cast<uint64_t *>(sm + 2 * DG2_STAGE);   // full[2], empty[2], tfull
  uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + 2 * DG2_STAGE + 64);
  volatile int *sfail = reinterpret_cast<volatile int *>(sm + 2 * DG2_STAGE + 72);
  auto full = [&](int st) { return smem_u32(&bars[st]); };
  auto empty = [&](int st) { return smem_u32(&bars[2 + st]); };
  const uint32_t tfull = smem_u32(&bars[4]);
  if (t == 0) {
    for (int b = 0; b < 5; ++b) mbar_init(smem_u32(&bars[b]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *sfail = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(DG_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;

  auto load = [&](int i) {   // thread 0: sub-block i into stage i & 1
    const int st = i & 1;
    const uint32_t sa = base + st * DG2_STAGE, sb = sa + DG_S * DG2_ASLAB;
    dg2_arrive_tx(full(st), DG2_STAGE);
    dg2_tma3(sa, &mapA, kfirst + i * DG2_SK, i0, full(st));
    dg2_tma3(sb, &mapB, kfirst + i * DG2_SK, j0, full(st));
  };
  int next_load = 0, consumed = 0;   // thread 0: sub-blocks loaded / whose copies were waited for
  if (t == 0) {
    for (; next_load < 2 && next_load < nsub; ++next_load) load(next_load);
  }
  const int quad = warp & 3, half = warp >> 2;
  long long acc[32];
#pragma unroll
  for (int c = 0; c < 32; ++c) acc[c] = 0;
  for (int w0 = 0, win = 0; w0 < nsub; w0 += DG2_WIN, ++win) {
    const int w1 = min(nsub, w0 + DG2_WIN);
    if (t == 0) {
      for (int i = w0; i < w1 && !*sfail; ++i) {
        if (!mbar_wait(full(i & 1), (uint32_t)((i >> 1) & 1))) {
          *sfail = 1;
          break;
        }
        consumed = i + 1;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t sa = base + (i & 1) * DG2_STAGE, sb = sa + DG_S * DG2_ASLAB;
        const uint64_t da0 = dg2_sdesc(sa), db0 = dg2_sdesc(sb);
#pragma unroll
        for (int g = 0; g < DG_S; ++g)
#pragma unroll
          for (int s = 0; s <= g; ++s)
#pragma unroll
            for (int kk = 0; kk < DG2_SK / 16; ++kk)
              tc_mma(tmem + (uint32_t)(g * DG_BN), da0 + (uint64_t)((s * DG2_ASLAB + kk * 32) >> 4),
                     db0 + (uint64_t)(((g - s) * DG2_BSLAB + kk * 32) >> 4), dg_idesc(),
                     (i > w0 || s > 0 || kk > 0) ? 1u : 0u);
        tc_commit(empty(i & 1));
        if (next_load == i + 1 && next_load < nsub) {
          // the stage of sub-block i + 1 held sub-block i - 1: free once its MMAs completed
          if (i >= 1 && !mbar_wait(empty((i - 1) & 1), (uint32_t)(((i - 1) >> 1) & 1))) {
            *sfail = 1;
            break;
          }
          load(next_load++);
        }
      }
      tc_commit(tfull);   // arrives once every MMA issued so far has completed
    }
    if (!mbar_wait(tfull, (uint32_t)(win & 1))) *sfail = 1;
    __syncthreads();
    if (*sfail) break;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // the window's last sub-block is done: its stage takes the sub-block after next
    if (t == 0 && next_load == w1 + 1 && next_load < nsub) load(next_load++);
    const uint32_t tlane = tmem + ((uint32_t)(quad * 32) << 16);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
#pragma unroll
      for (int g = 0; g < DG_S; g += 2) {
        uint32_t va[16], vb[16];
        tc_ld16(tlane + (uint32_t)(g * DG_BN + half * 32 + h * 16), va);
        tc_ld16(tlane + (uint32_t)((g + 1) * DG_BN + half * 32 + h * 16), vb);
        tc_wait_ld2x16(va, vb);
        const int sh = 7 * (DG_S - 2 - g) - R;
#pragma unroll
        for (int c = 0; c < 16; ++c) {
          const unsigned ga = (unsigned)__float2int_rn(__uint_as_float(va[c]));
          const unsigned gb = (unsigned)__float2int_rn(__uint_as_float(vb[c]));
          const int p = (int)((ga << 7) + gb);   // |2^7 G_g + G_{g+1}| < 2^31
          long long &a = acc[h * 16 + c];
          if (sh >= 0) a += (long long)p << sh;
          else a += (long long)((p + (1 << (-sh - 1))) >> (-sh));
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();   // TMEM free for the next window
  }
  const bool failed = *sfail != 0;
  if (failed && t == 0) {
    // copies still in flight: wait (bounded) for each before the shared memory goes away
    for (int i = consumed; i < next_load; ++i) mbar_wait(full(i & 1), (uint32_t)((i >> 1) & 1));
  }
  if (!failed && P != nullptr) {
    long long *Pz = P + (size_t)blockIdx.z * Mp * Np;
    const int row = i0 + quad * 32 + lane;
#pragma unroll
    for (int c = 0; c < 32; ++c) Pz[row + (size_t)(j0 + half * 32 + c) * Mp] = acc[c];
  } else if (!failed) {
    const int row = i0 + quad * 32 + lane;
    if (row < m) {
      const unsigned long long ma = rmaxA[row];
      const int ea = dg_row_exp(ma) - 61 + R;
      const bool bad_a = (ma >> 52) >= 2047ull;
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        const int col = j0 + half * 32 + c;
        if (col < n && (!(flags & kCLower) || row >= col)) {
          const unsigned long long mb = rmaxB[col];
          double x = ldexp((double)acc[c], ea + dg_row_exp(mb));
          if (bad_a || (mb >> 52) >= 2047ull) x = __longlong_as_double(0x7FF8000000000000ll);
          x *= alpha;
          double *cp = C + row + (size_t)col * ldc;
          if (beta != 0.0) x = fma(beta, *cp, x);
          *cp = x;
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(DG_TMEM_COLS) : "memory");
  }
  if (t == 0 && failed) atomicExch(err, 1);
}

// C = alpha 2^(EA_i + EB_j - 61 + R) sum_z P[z] + beta C over the elements a split-K product computed
// (integer sums: the result does not depend on the split).
__global__ void dg_splitk_reduce(int m, int n, int Mp, int Np, int splits, const long long *__restrict__ P,
                                 const unsigned long long *rmaxA, const unsigned long long *rmaxB, int R,
                                 double alpha, double beta, double *C, int ldc, int lowerC) {
  const size_t total = (size_t)m * n;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
    const int row = (int)(idx % m), col = (int)(idx / m);
    if (lowerC && row < col) continue;
    long long v = 0;
    for (int z = 0; z < splits; ++z) v += P[(size_t)z * Mp * Np + row + (size_t)col * Mp];
    const unsigned long long ma = rmaxA[row], mb = rmaxB[col];
    double x = ldexp((double)v, dg_row_exp(ma) + dg_row_exp(mb) - 61 + R);
    if ((ma >> 52) >= 2047ull || (mb >> 52) >= 2047ull) x = __longlong_as_double(0x7FF8000000000000ll);
    x *= alpha;
    double *cp = C + row + (size_t)col * ldc;
    if (beta != 0.0) x = fma(beta, *cp, x);
    *cp = x;
  }
}

// ------------------------------------------------------------------------------ host side
thread_local bool g_tc_dgemm = false;   // gemm<double> routes here while set (calling thread only)
std::atomic<bool> g_tc_dgemm_mixed{true};   // dftbgpu_set_fp64_emulation
std::atomic<int> g_dg_kernel{0};            // 0: single-stage kernel, 1: pipelined TMA kernel
constexpr int kDgSMs = 148;   // CTAs in flight (one per SM; GB300 has 152, a few may be taken)
// scratch of this thread on the current device: digit slabs, row maxima, split-K partials
static thread_local ThreadScratch t_dg;
enum { kDgSlabs = 0, kDgRmax = 1, kDgPart = 2 };

static int dg_round_up(int x, int q) { return (x + q - 1) / q * q; }

static int dg_ensure(DeviceScratch &d, size_t ws_elems, size_t rmax_elems) {
  int rc = scratch_reserve(d.buf[kDgSlabs], ws_elems * sizeof(__nv_bfloat16));
  if (rc == 0) rc = scratch_reserve(d.buf[kDgRmax], rmax_elems * sizeof(unsigned long long));
  if (rc == 0 && !d.err) {
    rc = scratch_err(d);
    if (rc == 0) rc = (int)cudaFuncSetAttribute(dg_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, DG_SMEM);
    if (rc == 0)
      rc = (int)cudaFuncSetAttribute(dg_gemm_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, DG2_SMEM);
  }
  return rc;
}

// 3D tensor map over packed digit slabs (K innermost, then rows, then the eight slabs) with a box of
// 32 K x box_rows rows x 8 slabs and the 64-byte swizzle; false if the driver cannot encode it.
static bool dg_slab_map(CUtensorMap *map, const __nv_bfloat16 *slabs, int rows, int Kp, int box_rows) {
  auto enc = tensor_map_encoder();
  if (enc == nullptr) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)rows, (cuuint64_t)DG_S};
  const cuuint64_t strides[2] = {(cuuint64_t)Kp * 2, (cuuint64_t)rows * Kp * 2};
  const cuuint32_t box[3] = {(cuuint32_t)DG2_SK, (cuuint32_t)box_rows, (cuuint32_t)DG_S}, es[3] = {1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void *)slabs, dims, strides, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// K-splits for a product with few output tiles: enough CTAs to fill the GPU, at least four K-blocks
// per split, at most 16 splits.
static int dg_splits(int m, int n, int k) {
  const long long tiles = (long long)ceil_div(m, DG_BM) * ceil_div(n, DG_BN);
  const int nkb = ceil_div(std::max(k, 1), DG_BK);
  if (tiles >= kDgSMs || nkb < 8) return 1;
  long long sp = (kDgSMs + tiles - 1) / tiles;
  sp = std::min<long long>(sp, nkb / 4);
  sp = std::min<long long>(sp, 16);
  return (int)std::max<long long>(sp, 1);
}

double tc_dgemm_estimate_s(int m, int n, int k) {
  const int sp = dg_splits(m, n, k);
  const double tiles = (double)ceil_div(m, DG_BM) * ceil_div(n, DG_BN) * sp;
  const double waves = std::ceil(tiles / kDgSMs);
  const double kb = std::ceil((double)ceil_div(std::max(k, 1), DG_BK) / sp);
  return waves * kb * 5e-6 + (sp > 1 ? 20e-6 : 15e-6);
}

int tc_dgemm_reserve(int m, int n, int k) {
  const size_t Mp = (size_t)dg_round_up(m, DG_BM), Np = (size_t)dg_round_up(n, DG_BN),
               Kp = (size_t)dg_round_up(std::max(k, 1), DG_BK);
  return dg_ensure(t_dg.current(), (size_t)DG_S * (Mp + Np) * Kp, Mp + Np);
}

int tc_dgemm(cudaStream_t s, char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda,
             const double *B, int ldb, double beta, double *C, int ldc, int flags) {
  if (m <= 0 || n <= 0) return 0;
  const int Mp = dg_round_up(m, DG_BM), Np = dg_round_up(n, DG_BN), Kp = dg_round_up(std::max(k, 1), DG_BK);
  DeviceScratch &ds = t_dg.current();
  int rc = dg_ensure(ds, (size_t)DG_S * ((size_t)Mp + (size_t)Np) * Kp, (size_t)Mp + Np);
  if (rc != 0) return rc;
  __nv_bfloat16 *PA = static_cast<__nv_bfloat16 *>(ds.buf[kDgSlabs].p), *PB = PA + (size_t)DG_S * Mp * Kp;
  unsigned long long *rA = static_cast<unsigned long long *>(ds.buf[kDgRmax].p), *rB = rA + Mp;
  const bool TA = (ta == 'T' || ta == 't'), TB = (tb == 'T' || tb == 't');
  // op(A)(r, k) and op(B)^T(j, k) as strided views; structural zeros from the triangular flags
  const long long ars = TA ? lda : 1, aks = TA ? 1 : lda;
  const long long brs = TB ? 1 : ldb, bks = TB ? ldb : 1;
  const int amask = (flags & kALower) ? 1 : ((flags & kAUpper) ? 2 : 0);
  const int bmask = (flags & kBLower) ? 2 : ((flags & kBUpper) ? 1 : 0);
  rc = (int)cudaMemsetAsync(rA, 0, ((size_t)Mp + Np) * sizeof(unsigned long long), s);
  if (rc != 0) return rc;
  const int kcm = std::max(1, ceil_div(k, kDgPackChunk)), kcp = ceil_div(Kp, kDgPackChunk);
  dg_rowmax_kernel<<<dim3(Mp / 32, kcm), 256, 0, s>>>(m, k, A, ars, aks, amask, rA);
  dg_rowmax_kernel<<<dim3(Np / 32, kcm), 256, 0, s>>>(n, k, B, brs, bks, bmask, rB);
  dg_pack_kernel<<<dim3(Mp / 32, kcp), 256, 0, s>>>(m, k, A, ars, aks, amask, Kp, (size_t)Mp * Kp, PA, rA);
  dg_pack_kernel<<<dim3(Np / 32, kcp), 256, 0, s>>>(n, k, B, brs, bks, bmask, Kp, (size_t)Np * Kp, PB, rB);
  int R = 0;
  while ((1 << (R + 1)) < Kp) ++R;   // R = ceil(log2 Kp) - 1
  const int splits = dg_splits(m, n, k);
  long long *Pp = nullptr;
  int kb_split = 0;
  if (splits > 1) {
    rc = scratch_reserve(ds.buf[kDgPart], (size_t)splits * Mp * Np * sizeof(long long));
    if (rc != 0) return rc;
    Pp = static_cast<long long *>(ds.buf[kDgPart].p);
    kb_split = ceil_div(Kp / DG_BK, splits);
  }
  CUtensorMap mapA, mapB;
  if (g_dg_kernel.load() == 1 && dg_slab_map(&mapA, PA, Mp, Kp, DG_BM) && dg_slab_map(&mapB, PB, Np, Kp, DG_BN))
    dg_gemm_tma_kernel<<<dim3(Mp / DG_BM, Np / DG_BN, splits), DG_THREADS, DG2_SMEM, s>>>(
        mapA, mapB, m, n, Kp, Mp, Np, rA, rB, R, alpha, beta, C, ldc, flags, ds.err, Pp, kb_split);
  else
    dg_gemm_kernel<<<dim3(Mp / DG_BM, Np / DG_BN, splits), DG_THREADS, DG_SMEM, s>>>(
        m, n, Kp, Mp, Np, PA, PB, rA, rB, R, alpha, beta, C, ldc, flags, ds.err, Pp, kb_split);
  count_launch(5);
  if (Pp) {
    const int rb = (int)std::min<long long>(((long long)m * n + 255) / 256, 152 * 8);
    dg_splitk_reduce<<<rb, 256, 0, s>>>(m, n, Mp, Np, splits, Pp, rA, rB, R, alpha, beta, C, ldc,
                                        (flags & kCLower) ? 1 : 0);
    count_launch();
  }
  return (int)cudaGetLastError();
}

int tc_dgemm_error() { return scratch_take_err(t_dg.current()); }

}  // namespace dg
