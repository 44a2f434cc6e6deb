// Reductions and a bounded grid barrier shared by the cooperative kernels (tridiagonalisation
// panels in linalg.cu, the panel QR and bulge chasing of the two-stage reduction in twostage.cu).
#pragma once
#include "common.cuh"

namespace dg {

constexpr unsigned kBarrierSpinLimit = 1u << 24;   // polls (about a second) before a barrier gives up

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int NT, typename T>
__device__ T block_sum(T v, T *sh) {
  v = warp_sum(v);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  T r = T(0);
  if (threadIdx.x < 32) {
    r = (threadIdx.x < NT / 32) ? sh[threadIdx.x] : T(0);
    r = warp_sum(r);
    if (threadIdx.x == 0) sh[0] = r;
  }
  __syncthreads();
  r = sh[0];
  __syncthreads();
  return r;
}

// Grid barrier state, zeroed once per reduction: a monotonic arrival counter (barrier number e of
// the reduction completes when count reaches (e + 1) * CTAs) and an error word.
struct GridBar {
  unsigned count, pad0;
  int err, pad1;
};

// Grid barrier for a cooperative launch (all CTAs co-resident): one release-ordered arrival per CTA
// (the CTA's writes before the barrier become visible with it), then acquire polls until every
// CTA of this barrier number has arrived. Bounded: after kBarrierSpinLimit polls it records an
// error and stops waiting; once an error is recorded no barrier waits any more, so a broken launch
// ends quickly with the error set.
__device__ __forceinline__ unsigned grid_load_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void grid_sync(GridBar *b, unsigned nb, unsigned &epoch) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile int *verr = &b->err;
    if (*verr == 0) {
      asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(&b->count), "r"(1u) : "memory");
      const unsigned target = (epoch + 1u) * nb;
      unsigned it = 0;
      while ((int)(grid_load_acquire(&b->count) - target) < 0) {
        if (++it > kBarrierSpinLimit) {
          atomicExch(&b->err, 1);
          break;
        }
      }
    }
  }
  ++epoch;
  __syncthreads();
}

// The same barrier for a launch whose grid size may differ from that of the earlier launches on the
// same counter: the counter stood at `base` when the launch started, so barrier e of the launch
// completes when it reaches base + (e + 1) * nb. Thread 0 runs before_arrive() after the entry
// __syncthreads and before its arrival (the release orders what it writes before the arrival).
template <class F>
__device__ __forceinline__ void grid_sync_base(GridBar *b, unsigned nb, unsigned base, unsigned &e, F before_arrive) {
  __syncthreads();
  if (threadIdx.x == 0) {
    before_arrive();
    volatile int *verr = &b->err;
    if (*verr == 0) {
      asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(&b->count), "r"(1u) : "memory");
      const unsigned target = base + (e + 1u) * nb;
      unsigned it = 0;
      while ((int)(grid_load_acquire(&b->count) - target) < 0) {
        if (++it > kBarrierSpinLimit) {
          atomicExch(&b->err, 1);
          break;
        }
      }
    }
  }
  ++e;
  __syncthreads();
}

}  // namespace dg
